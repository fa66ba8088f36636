// Host check of the eight-wide BVH: builds the binary SAH tree and its eight-wide collapse for
// the triangles in a binary file, then traces random rays with the device traversal code
// (wide_trav.h, compiled here for the CPU) and with brute force over every triangle.
//
//   wide_check <scene.bin> <num_rays> <seed>
// scene.bin: uint32 nv, uint32 nt, float pos[3 nv], uint32 tris[3 nt] (global vertex indices).
// Prints one line of counts; exit status 0 when every closest hit has the brute-force distance
// bit for bit (and the same triangle or one at exactly that distance) and every any-hit answer
// agrees.
#include "bvh.h"
#include "bvh_wide.h"
#include "wide_trav.h"

#include <vector_functions.h>

#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

using namespace e8g;

int main(int argc, char **argv) {
    if (argc < 4)
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
    uint32_t nrays = static_cast<uint32_t>(std::atoi(argv[2]));
    std::mt19937 rng(static_cast<uint32_t>(std::atoi(argv[3])));

    bvh_build_opts o; // the product defaults
    flat_bvh b = build_bvh(pos.data(), tris.data(), nt, o);
    float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f}, max_abs = 0;
    for (uint32_t v = 0; v < nv; v++)
        for (int a = 0; a < 3; a++) {
            lo[a] = std::min(lo[a], pos[3 * v + a]);
            hi[a] = std::max(hi[a], pos[3 * v + a]);
            max_abs = std::max(max_abs, std::fabs(pos[3 * v + a]));
        }
    wide_bvh w = collapse_wide(b, pos.data(), tris.data(), max_abs * 2.0f);
    // triangle records in wide order, and in global order for brute force
    auto record = [&](uint32_t t, float4 *r) {
        float const *v0 = &pos[3 * tris[3 * t]], *v1 = &pos[3 * tris[3 * t + 1]], *v2 = &pos[3 * tris[3 * t + 2]];
        float id;
        std::memcpy(&id, &t, 4);
        r[0] = make_float4(v0[0], v0[1], v0[2], id);
        r[1] = make_float4(v1[0] - v0[0], v1[1] - v0[1], v1[2] - v0[2], 0.0f);
        r[2] = make_float4(v2[0] - v0[0], v2[1] - v0[1], v2[2] - v0[2], 0.0f);
    };
    std::vector<float4> rec(3 * static_cast<size_t>(nt)), grec(3 * static_cast<size_t>(nt));
    for (uint32_t k = 0; k < w.tri_order.size(); k++)
        record(w.tri_order[k], &rec[3 * k]);
    for (uint32_t t = 0; t < nt; t++)
        record(t, &grec[3 * t]);
    WideView W{reinterpret_cast<uint4 const *>(w.nodes.data()), rec.data(), w.num_nodes};
    // level boundaries (the refit's launches): one per level, increasing, ending at the node
    // count, and every interior child of a level-L node in level L + 1
    uint64_t bad_levels = 0;
    if (w.level_start.size() != w.max_depth + 1 || w.level_start.empty() || w.level_start[0] != 0 ||
        w.level_start.back() != w.num_nodes)
        bad_levels++;
    for (uint32_t L = 0; !bad_levels && L < w.max_depth; L++) {
        if (w.level_start[L] >= w.level_start[L + 1])
            bad_levels++;
        for (uint32_t i = w.level_start[L]; i < w.level_start[L + 1]; i++) {
            uint32_t const *nd = &w.nodes[kWideWords * static_cast<size_t>(i)];
            uint32_t imask = nd[3] >> 24, nch = static_cast<uint32_t>(__builtin_popcount(imask));
            if (nch && (L + 2 > w.max_depth || nd[4] < w.level_start[L + 1] || nd[4] + nch > w.level_start[L + 2]))
                bad_levels++;
        }
    }

    std::uniform_real_distribution<float> U(0.0f, 1.0f);
    uint64_t bad_t = 0, bad_tri = 0, bad_any = 0, hits = 0, visits = 0, tested = 0;
    uint32_t stk[2 * kWideStack];
    for (uint32_t r = 0; r < nrays; r++) {
        float3 org, dir;
        if (r % 4 == 3) { // a ray from a vertex (surface origins, shared edges)
            uint32_t v = static_cast<uint32_t>(U(rng) * nv) % nv;
            org = make_float3(pos[3 * v], pos[3 * v + 1], pos[3 * v + 2]);
        } else {
            org = make_float3(lo[0] + (hi[0] - lo[0]) * (1.2f * U(rng) - 0.1f), lo[1] + (hi[1] - lo[1]) * (1.2f * U(rng) - 0.1f),
                              lo[2] + (hi[2] - lo[2]) * (1.2f * U(rng) - 0.1f));
        }
        float dx = 2 * U(rng) - 1, dy = 2 * U(rng) - 1, dz = 2 * U(rng) - 1;
        if (r % 8 == 7 && nt) { // a grazing ray: from a point of a triangle, along its plane
            uint32_t t = static_cast<uint32_t>(U(rng) * nt) % nt;
            float const *v0 = &pos[3 * tris[3 * t]], *v1 = &pos[3 * tris[3 * t + 1]], *v2 = &pos[3 * tris[3 * t + 2]];
            float u = U(rng), v = U(rng) * (1 - u), a = U(rng) - 0.5f, b = U(rng) - 0.5f;
            org = make_float3(v0[0] + u * (v1[0] - v0[0]) + v * (v2[0] - v0[0]),
                              v0[1] + u * (v1[1] - v0[1]) + v * (v2[1] - v0[1]),
                              v0[2] + u * (v1[2] - v0[2]) + v * (v2[2] - v0[2]));
            dx = a * (v1[0] - v0[0]) + b * (v2[0] - v0[0]);
            dy = a * (v1[1] - v0[1]) + b * (v2[1] - v0[1]);
            dz = a * (v1[2] - v0[2]) + b * (v2[2] - v0[2]);
        }
        if (r % 16 == 5)
            dx = dy = 0.0f; // axis-aligned rays
        if (r % 16 == 9)
            dy = -0.0f;
        float n = std::sqrt(dx * dx + dy * dy + dz * dz);
        if (!(n > 0))
            dz = n = 1.0f;
        dir = make_float3(dx / n, dy / n, dz / n);
        // brute force closest on [1e-4, 1000], strict < in index order
        Hit bf{INFINITY, 0xFFFFFFFFu, 0, 0};
        for (uint32_t t = 0; t < nt; t++) {
            float t0, b1, b2;
            if (hd_tri_test(org, dir, grec[3 * t], grec[3 * t + 1], grec[3 * t + 2], 1e-4f, 1000.0f, t0, b1, b2) &&
                t0 < bf.t) {
                bf.t = t0;
                bf.tri = t;
            }
        }
        uint32_t cn = 0, ct = 0;
        Hit h = wide_trace(W, org, dir, 1e-4f, 1000.0f, false, stk, 1, &cn, &ct);
        visits += cn;
        tested += ct;
        if (bf.tri != 0xFFFFFFFFu)
            hits++;
        uint32_t a, b2;
        std::memcpy(&a, &h.t, 4);
        std::memcpy(&b2, &bf.t, 4);
        if (a != b2 && !(bf.tri == 0xFFFFFFFFu && h.tri == 0xFFFFFFFFu)) {
            bad_t++;
        } else if (h.tri != bf.tri) {
            float t0, b1, bb2;
            bool same = h.tri < nt &&
                        hd_tri_test(org, dir, grec[3 * h.tri], grec[3 * h.tri + 1], grec[3 * h.tri + 2], 1e-4f, 1000.0f, t0, b1, bb2) &&
                        t0 == bf.t;
            if (!same)
                bad_tri++;
        }
        // any hit on [1e-4, tmax]
        float tmax = 0.05f + 3.0f * U(rng) * (hi[0] - lo[0] + hi[1] - lo[1] + hi[2] - lo[2]) / 3.0f;
        bool bfa = false;
        for (uint32_t t = 0; t < nt && !bfa; t++) {
            float t0, b1, bb2;
            bfa = hd_tri_test(org, dir, grec[3 * t], grec[3 * t + 1], grec[3 * t + 2], 1e-4f, tmax, t0, b1, bb2);
        }
        bool wa = wide_trace(W, org, dir, 1e-4f, tmax, true, stk, 1, nullptr, nullptr).tri != 0xFFFFFFFFu;
        if (wa != bfa)
            bad_any++;
    }
    std::printf("{\"tris\": %u, \"binary_nodes\": %u, \"wide_nodes\": %u, \"wide_depth\": %u, \"ok\": %d, "
                "\"rays\": %u, \"hits\": %llu, \"bad_t\": %llu, \"bad_tri\": %llu, \"bad_any\": %llu, "
                "\"visits_per_ray\": %.3f, \"tris_per_ray\": %.3f, \"bad_levels\": %llu}\n",
                nt, b.num_nodes, w.num_nodes, w.max_depth, w.ok ? 1 : 0, nrays, (unsigned long long)hits,
                (unsigned long long)bad_t, (unsigned long long)bad_tri, (unsigned long long)bad_any,
                nrays ? double(visits) / nrays : 0.0, nrays ? double(tested) / nrays : 0.0,
                (unsigned long long)bad_levels);
    return (bad_t || bad_tri || bad_any || bad_levels || !w.ok) ? 1 : 0;
}
