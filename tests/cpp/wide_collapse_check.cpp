// Host collapse of a given binary SAH tree (the library's bvh_wide.cpp), for comparison with the
// device collapse of the same tree.
//
//   wide_collapse_check <scene.bin> <tree.bin> <max_abs> <out.bin>
// scene.bin: uint32 nv, uint32 nt, float pos[3 nv], uint32 tris[3 nt] (global vertex indices).
// tree.bin: uint32 num_nodes, float lo[4 num_nodes], float hi[4 num_nodes], uint32 tri_order[nt]
// (the layout e8g_bvh_read returns, with the order taken from the triangle records).
// out.bin: uint32 ok, uint32 num_nodes, uint32 nodes[24 num_nodes], uint32 tri_order[nt].
#include "bvh.h"
#include "bvh_boxes.h"
#include "bvh_wide.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

using namespace e8g;

int main(int argc, char **argv) {
    if (argc < 5)
        return 2;
    FILE *f = std::fopen(argv[1], "rb");
    if (!f)
        return 2;
    uint32_t nv = 0, nt = 0;
    if (std::fread(&nv, 4, 1, f) != 1 || std::fread(&nt, 4, 1, f) != 1)
        return 2;
    std::vector<float> pos(3 * static_cast<size_t>(nv));
    std::vector<uint32_t> tris(3 * static_cast<size_t>(nt));
    if (std::fread(pos.data(), 4, pos.size(), f) != pos.size() || std::fread(tris.data(), 4, tris.size(), f) != tris.size())
        return 2;
    std::fclose(f);
    f = std::fopen(argv[2], "rb");
    if (!f)
        return 2;
    flat_bvh b;
    if (std::fread(&b.num_nodes, 4, 1, f) != 1)
        return 2;
    b.lo.resize(4 * static_cast<size_t>(b.num_nodes));
    b.hi.resize(4 * static_cast<size_t>(b.num_nodes));
    b.tri_order.resize(nt);
    if (std::fread(b.lo.data(), 4, b.lo.size(), f) != b.lo.size() || std::fread(b.hi.data(), 4, b.hi.size(), f) != b.hi.size() ||
        std::fread(b.tri_order.data(), 4, nt, f) != nt)
        return 2;
    std::fclose(f);
    // eps of the scene box over the triangles, as both builders take it
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t t = 0; t < nt; t++)
        for (int v = 0; v < 3; v++)
            for (int a = 0; a < 3; a++) {
                float x = pos[3 * static_cast<size_t>(tris[3 * static_cast<size_t>(t) + v]) + a];
                lo[a] = x < lo[a] ? x : lo[a];
                hi[a] = hi[a] < x ? x : hi[a];
            }
    b.eps = scene_eps(lo, hi);
    wide_bvh w = collapse_wide(b, pos.data(), tris.data(), std::strtof(argv[3], nullptr));
    f = std::fopen(argv[4], "wb");
    if (!f)
        return 2;
    uint32_t head[2] = {w.ok ? 1u : 0u, w.num_nodes};
    std::fwrite(head, 4, 2, f);
    std::fwrite(w.nodes.data(), 4, w.nodes.size(), f);
    std::fwrite(w.tri_order.data(), 4, w.tri_order.size(), f);
    std::fclose(f);
    return 0;
}
