// Incremental scene updates on the device: trimesh::transform of one mesh and the refit of the
// tree after its vertices moved (no counterpart in the reference, which rebuilds the whole tree
// on every commit: bvh_path_space_layout::commit, pathspace.cpp:292-328).
//
// A refit keeps the tree's topology and recomputes every box from the triangles below it, with
// the arithmetic of the host build (bvh_boxes.h): each box is the exact union of its triangles'
// vertices pushed out by |v| * 1e-6 + eps, eps from the scene's exact box, and eight-wide nodes
// re-quantize their children on a fresh grid. One pass goes bottom-up: a thread starts at every
// leaf-holding node, and at each parent the last child to arrive (an atomic counter per node)
// carries on upwards with the union of the children's exact boxes; no thread ever waits. The
// eight-wide tree, breadth first and at most 16 levels deep, is refitted one level per launch.
#include "bvh_boxes.h"
#include "bvh_wide.h"
#include "launch.h"
#include "refit.h"

#include <cstdint>
#include <cstring>

namespace e8g {
namespace {

constexpr int kRefitBlock = 256;

// Order-preserving map of floats to unsigned integers, so atomicMin / atomicMax on the integers
// give the float minimum / maximum.
__device__ __forceinline__ uint32_t ord_of(float f) {
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float of_ord(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

// Arrival at a parent: release of this thread's writes, acquire of the siblings' (their arrivals
// are earlier in the counter's modification order).
__device__ __forceinline__ uint32_t arrive(uint32_t *counter) {
    uint32_t old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;" : "=r"(old) : "l"(counter) : "memory");
    return old;
}

// Block-wide min / max of `n` values per thread into red[...] with one atomic per block and word.
template <int N, bool MAX>
__device__ __forceinline__ void block_reduce(uint32_t (&v)[N], uint32_t *red) {
    __shared__ uint32_t sh[kRefitBlock / 32][N];
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < N; k++) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            uint32_t x = __shfl_xor_sync(0xFFFFFFFFu, v[k], o);
            v[k] = MAX ? max(v[k], x) : min(v[k], x);
        }
        if (lane == 0)
            sh[warp][k] = v[k];
    }
    __syncthreads();
    if (threadIdx.x < N) {
        uint32_t r = sh[0][threadIdx.x];
        for (int w = 1; w < kRefitBlock / 32; w++)
            r = MAX ? max(r, sh[w][threadIdx.x]) : min(r, sh[w][threadIdx.x]);
        if (MAX)
            atomicMax(&red[threadIdx.x], r);
        else
            atomicMin(&red[threadIdx.x], r);
    }
}

__global__ void k_refit_init(uint32_t *red) {
    int i = threadIdx.x;
    if (i < kRefitRedWords) // minima start at the largest key, maxima and |max| at 0
        red[i] = (i < 3 || (i >= 6 && i < 9)) ? 0xFFFFFFFFu : 0u;
}

// Box over all vertices (the path space's aabb) and the largest |coordinate|.
__global__ void __launch_bounds__(kRefitBlock) k_refit_verts(float4 const *vpos, uint32_t nv, uint32_t *red) {
    uint32_t mn[3] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu};
    uint32_t mx[4] = {0, 0, 0, 0};
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x) {
        float4 p = vpos[v];
        float c[3] = {p.x, p.y, p.z};
#pragma unroll
        for (int a = 0; a < 3; a++) {
            mn[a] = min(mn[a], ord_of(c[a]));
            mx[a] = max(mx[a], ord_of(c[a]));
            mx[3] = max(mx[3], __float_as_uint(fabsf(c[a])));
        }
    }
    block_reduce<3, false>(mn, red + 6);
    __syncthreads();
    block_reduce<4, true>(mx, red + 9);
}

// Triangle records (v0 | id, v1 - v0, v2 - v0) from the current vertices, and the exact box of
// all triangles (the scene box the boxes' eps derives from).
__global__ void __launch_bounds__(kRefitBlock) k_refit_tris(float4 *tri, uint4 const *tidx, float4 const *vpos,
                                                             uint32_t nt, uint32_t *red, float4 *tlo, float4 *thi) {
    uint32_t mn[3] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu};
    uint32_t mx[3] = {0, 0, 0};
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < nt; k += gridDim.x * blockDim.x) {
        float w = tri[3 * static_cast<size_t>(k)].w;
        uint4 g = tidx[__float_as_uint(w)];
        float4 p0 = vpos[g.x], p1 = vpos[g.y], p2 = vpos[g.z];
        tri[3 * static_cast<size_t>(k)] = make_float4(p0.x, p0.y, p0.z, w);
        tri[3 * static_cast<size_t>(k) + 1] = make_float4(p1.x - p0.x, p1.y - p0.y, p1.z - p0.z, 0.0f);
        tri[3 * static_cast<size_t>(k) + 2] = make_float4(p2.x - p0.x, p2.y - p0.y, p2.z - p0.z, 0.0f);
        tlo[k] = make_float4(fminf(fminf(p0.x, p1.x), p2.x), fminf(fminf(p0.y, p1.y), p2.y),
                             fminf(fminf(p0.z, p1.z), p2.z), 0.0f);
        thi[k] = make_float4(fmaxf(fmaxf(p0.x, p1.x), p2.x), fmaxf(fmaxf(p0.y, p1.y), p2.y),
                             fmaxf(fmaxf(p0.z, p1.z), p2.z), 0.0f);
        float c[3][3] = {{p0.x, p0.y, p0.z}, {p1.x, p1.y, p1.z}, {p2.x, p2.y, p2.z}};
#pragma unroll
        for (int v = 0; v < 3; v++)
#pragma unroll
            for (int a = 0; a < 3; a++) {
                mn[a] = min(mn[a], ord_of(c[v][a]));
                mx[a] = max(mx[a], ord_of(c[v][a]));
            }
    }
    block_reduce<3, false>(mn, red);
    __syncthreads();
    block_reduce<3, true>(mx, red + 3);
}

__device__ __forceinline__ float scene_eps_of(uint32_t const *red) {
    float lo[3], hi[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        lo[a] = of_ord(red[a]);
        hi[a] = of_ord(red[3 + a]);
    }
    return scene_eps(lo, hi);
}

// Exact box of the triangles at record positions [first, first + n), from their boxes.
__device__ __forceinline__ void range_box(float4 const *tlo, float4 const *thi, uint32_t first, uint32_t n,
                                          float lo[3], float hi[3]) {
    for (int a = 0; a < 3; a++) {
        lo[a] = INFINITY;
        hi[a] = -INFINITY;
    }
    for (uint32_t k = first; k < first + n; k++) {
        float4 a = __ldg(&tlo[k]), b = __ldg(&thi[k]);
        lo[0] = fminf(lo[0], a.x), hi[0] = fmaxf(hi[0], b.x);
        lo[1] = fminf(lo[1], a.y), hi[1] = fmaxf(hi[1], b.y);
        lo[2] = fminf(lo[2], a.z), hi[2] = fmaxf(hi[2], b.z);
    }
}

// ---------------------------------------------------------------- SAH child pairs ----

__global__ void k_parents_pairs(float4 const *nlo, float4 const *nhi, uint32_t nn, uint32_t *parent) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn || __float_as_uint(nhi[i].w) != 0)
        return;
    uint32_t link = __float_as_uint(nlo[i].w);
    parent[link] = i;
    parent[link + 1] = i;
}

__device__ __forceinline__ void store_pair_node(float4 *nlo, float4 *nhi, uint32_t n, float const lo[3],
                                                float const hi[3], float eps, float4 *ex_lo, float4 *ex_hi) {
    ex_lo[n] = make_float4(lo[0], lo[1], lo[2], 0.0f);
    ex_hi[n] = make_float4(hi[0], hi[1], hi[2], 0.0f);
    float lw = nlo[n].w, hw = nhi[n].w; // link and count stay
    nlo[n] = make_float4(inflate_lo(lo[0], eps), inflate_lo(lo[1], eps), inflate_lo(lo[2], eps), lw);
    nhi[n] = make_float4(inflate_hi(hi[0], eps), inflate_hi(hi[1], eps), inflate_hi(hi[2], eps), hw);
}

__global__ void __launch_bounds__(kRefitBlock)
    k_refit_pairs(float4 *nlo, float4 *nhi, uint32_t nn, float4 const *tlo, float4 const *thi, uint32_t const *parent,
                  uint32_t *counter, float4 *ex_lo, float4 *ex_hi, uint32_t const *red) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn)
        return;
    uint32_t count = __float_as_uint(nhi[i].w);
    if (count == 0)
        return;
    float eps = scene_eps_of(red);
    float lo[3], hi[3];
    range_box(tlo, thi, __float_as_uint(nlo[i].w), count, lo, hi);
    store_pair_node(nlo, nhi, i, lo, hi, eps, ex_lo, ex_hi);
    uint32_t n = parent[i];
    while (n != 0xFFFFFFFFu) {
        if (arrive(&counter[n]) == 0)
            return; // the sibling's thread finishes this node
        uint32_t c = __float_as_uint(nlo[n].w);
        float4 a0 = __ldcg(&ex_lo[c]), a1 = __ldcg(&ex_hi[c]);
        float4 b0 = __ldcg(&ex_lo[c + 1]), b1 = __ldcg(&ex_hi[c + 1]);
        lo[0] = fminf(a0.x, b0.x), lo[1] = fminf(a0.y, b0.y), lo[2] = fminf(a0.z, b0.z);
        hi[0] = fmaxf(a1.x, b1.x), hi[1] = fmaxf(a1.y, b1.y), hi[2] = fmaxf(a1.z, b1.z);
        store_pair_node(nlo, nhi, n, lo, hi, eps, ex_lo, ex_hi);
        n = parent[n];
    }
}

// ------------------------------------------------------------------- eight-wide ----

__device__ void refit_wide_node(uint4 *wn, uint32_t i, float4 const *tlo, float4 const *thi, float4 *ex_lo,
                                float4 *ex_hi, float eps, double step_min) {
    uint32_t w[kWideWords];
    uint4 *node = wn + 6 * static_cast<size_t>(i);
#pragma unroll
    for (int q = 0; q < 6; q++) {
        uint4 x = node[q];
        w[4 * q] = x.x, w[4 * q + 1] = x.y, w[4 * q + 2] = x.z, w[4 * q + 3] = x.w;
    }
    uint32_t imask = w[3] >> 24, base = w[4], tri_base = w[5], counts = w[20], leaves = w[21];
    float slo[8][3], shi[8][3];
    float nlo[3] = {INFINITY, INFINITY, INFINITY}, nhi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int s = 0; s < 8; s++) {
        float lo[3], hi[3];
        if (imask >> s & 1) {
            uint32_t c = base + __popc(imask & ((1u << s) - 1));
            float4 a = __ldcg(&ex_lo[c]), b = __ldcg(&ex_hi[c]);
            lo[0] = a.x, lo[1] = a.y, lo[2] = a.z, hi[0] = b.x, hi[1] = b.y, hi[2] = b.z;
        } else if (leaves >> s & 1) {
            uint32_t meta = (w[6 + (s >> 2)] >> (8 * (s & 3))) & 0xFFu;
            range_box(tlo, thi, tri_base + meta, (counts >> (4 * s)) & 0xFu, lo, hi);
        } else {
            for (int a = 0; a < 3; a++)
                slo[s][a] = shi[s][a] = 0.0f;
            continue;
        }
        for (int a = 0; a < 3; a++) {
            nlo[a] = fminf(nlo[a], lo[a]);
            nhi[a] = fmaxf(nhi[a], hi[a]);
            slo[s][a] = inflate_lo(lo[a], eps);
            shi[s][a] = inflate_hi(hi[a], eps);
        }
    }
    wide_quantize(slo, shi, imask | leaves, step_min, w);
    node[0] = make_uint4(w[0], w[1], w[2], w[3]);
    node[2] = make_uint4(w[8], w[9], w[10], w[11]);
    node[3] = make_uint4(w[12], w[13], w[14], w[15]);
    node[4] = make_uint4(w[16], w[17], w[18], w[19]);
    ex_lo[i] = make_float4(nlo[0], nlo[1], nlo[2], 0.0f);
    ex_hi[i] = make_float4(nhi[0], nhi[1], nhi[2], 0.0f);
}

// One level of the eight-wide tree (its nodes are contiguous: the layout is breadth first),
// after every deeper level: the children's exact boxes are final, so nothing waits or counts.
__global__ void __launch_bounds__(kRefitBlock)
    k_refit_wide_level(uint4 *wn, uint32_t first, uint32_t count, float4 const *tlo, float4 const *thi,
                       float4 *ex_lo, float4 *ex_hi, uint32_t const *red, float cam_abs) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count)
        return;
    float eps = scene_eps_of(red);
    double step_min = wide_step_min(fmaxf(__uint_as_float(red[12]), cam_abs));
    refit_wide_node(wn, first + k, tlo, thi, ex_lo, ex_hi, eps, step_min);
}

// ------------------------------------------------------------------ transform ----

__global__ void k_transform(float4 const *vpos0, float4 const *vnrm0, float4 *vpos, float4 *vnrm, XformArgs X) {
    uint32_t v = X.v_begin + blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= X.v_end)
        return;
    // mat * vec (tensor.h:425-433): each component summed from 0 over the columns in order
    float4 p = vpos0[v];
    float h[4] = {p.x, p.y, p.z, 1.0f}, o[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        float acc = 0.0f;
#pragma unroll
        for (int j = 0; j < 4; j++)
            acc = acc + X.m[4 * i + j] * h[j];
        o[i] = acc;
    }
    float inv_w = 1.0f / o[3]; // vec::cart (tensor.h:261-268)
    vpos[v] = make_float4(inv_w * o[0], inv_w * o[1], inv_w * o[2], 0.0f);
    float4 n = vnrm0[v];
    float hn[4] = {n.x, n.y, n.z, X.directions ? 0.0f : 1.0f};
#pragma unroll
    for (int i = 0; i < 4; i++) {
        float acc = 0.0f;
#pragma unroll
        for (int j = 0; j < 4; j++)
            acc = acc + X.n[4 * i + j] * hn[j];
        o[i] = acc;
    }
    if (X.directions) {
        vnrm[v] = make_float4(o[0], o[1], o[2], 0.0f);
    } else {
        float inv_wn = 1.0f / o[3];
        vnrm[v] = make_float4(inv_wn * o[0], inv_wn * o[1], inv_wn * o[2], 0.0f);
    }
}

inline int blocks_for(uint64_t n) { return n ? static_cast<int>((n + kRefitBlock - 1) / kRefitBlock) : 1; }

} // namespace

size_t refit_scratch_bytes(uint32_t nn, uint32_t nt) {
    return 4 * static_cast<size_t>(kRefitRedWords) + 32 * static_cast<size_t>(nn) + 8 * static_cast<size_t>(nn) +
           32 * static_cast<size_t>(nt) + 16;
}

RefitScratch refit_carve(void *base, uint32_t nn, uint32_t nt) {
    RefitScratch r;
    char *p = static_cast<char *>(base);
    r.red = reinterpret_cast<uint32_t *>(p);
    p += 4 * kRefitRedWords;
    r.ex_lo = reinterpret_cast<float4 *>(p);
    p += 16 * static_cast<size_t>(nn);
    r.ex_hi = reinterpret_cast<float4 *>(p);
    p += 16 * static_cast<size_t>(nn);
    r.parent = reinterpret_cast<uint32_t *>(p);
    p += 4 * static_cast<size_t>(nn);
    r.counter = reinterpret_cast<uint32_t *>(p);
    p += 4 * static_cast<size_t>(nn);
    p = reinterpret_cast<char *>((reinterpret_cast<uintptr_t>(p) + 15) & ~uintptr_t(15));
    r.tlo = reinterpret_cast<float4 *>(p);
    p += 16 * static_cast<size_t>(nt);
    r.thi = reinterpret_cast<float4 *>(p);
    return r;
}

void launch_refit_parents(DevScene const &S, RefitScratch const &R, cudaStream_t st) {
    uint32_t nn = S.nnodes;
    if (S.layout == 2) // the eight-wide refit goes level by level instead
        return;
    cudaMemsetAsync(R.parent, 0xFF, 4 * static_cast<size_t>(nn), st);
    k_parents_pairs<<<blocks_for(nn), kRefitBlock, 0, st>>>(S.nlo, S.nhi, nn, R.parent);
}

void launch_refit(DevScene const &S, RefitScratch const &R, uint32_t nv, float cam_abs, int grid_cap,
                  uint32_t const *wide_levels, uint32_t num_levels, cudaStream_t st) {
    uint32_t nn = S.nnodes, nt = S.ntris;
    float4 *tri = const_cast<float4 *>(S.tri);
    if (S.layout != 2)
        cudaMemsetAsync(R.counter, 0, 4 * static_cast<size_t>(nn), st);
    k_refit_init<<<1, 32, 0, st>>>(R.red);
    k_refit_verts<<<min(blocks_for(nv), grid_cap), kRefitBlock, 0, st>>>(S.vpos, nv, R.red);
    k_refit_tris<<<min(blocks_for(nt), grid_cap), kRefitBlock, 0, st>>>(tri, S.tidx, S.vpos, nt, R.red, R.tlo, R.thi);
    if (S.layout == 2) {
        for (uint32_t l = num_levels; l-- > 0;) { // deepest level first
            uint32_t first = wide_levels[l], count = wide_levels[l + 1] - wide_levels[l];
            if (count)
                k_refit_wide_level<<<blocks_for(count), kRefitBlock, 0, st>>>(const_cast<uint4 *>(S.wnodes), first,
                                                                              count, R.tlo, R.thi, R.ex_lo, R.ex_hi,
                                                                              R.red, cam_abs);
        }
    } else
        k_refit_pairs<<<blocks_for(nn), kRefitBlock, 0, st>>>(const_cast<float4 *>(S.nlo), const_cast<float4 *>(S.nhi),
                                                                nn, R.tlo, R.thi, R.parent, R.counter, R.ex_lo,
                                                                R.ex_hi, R.red);
}

namespace {
__global__ void k_interleave(float4 const *vpos, float4 const *vnrm, uint32_t nv, float4 *vtx) {
    uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv)
        return;
    float4 p = vpos[v], n = vnrm[v];
    vtx[2 * static_cast<size_t>(v)] = make_float4(p.x, p.y, p.z, n.x);
    vtx[2 * static_cast<size_t>(v) + 1] = make_float4(n.y, n.z, 0.0f, 0.0f);
}
} // namespace

void launch_interleave(float4 const *vpos, float4 const *vnrm, uint32_t nv, float4 *vtx, cudaStream_t st) {
    if (nv)
        k_interleave<<<blocks_for(nv), kRefitBlock, 0, st>>>(vpos, vnrm, nv, vtx);
}

void launch_vertex_bounds(float4 const *vpos, uint32_t nv, uint32_t *red, int grid_cap, cudaStream_t st) {
    k_refit_init<<<1, 32, 0, st>>>(red);
    k_refit_verts<<<min(blocks_for(nv), grid_cap), kRefitBlock, 0, st>>>(vpos, nv, red);
}

void launch_transform(float4 const *vpos0, float4 const *vnrm0, float4 *vpos, float4 *vnrm, XformArgs const &X,
                      cudaStream_t st) {
    if (X.v_end > X.v_begin)
        k_transform<<<blocks_for(X.v_end - X.v_begin), kRefitBlock, 0, st>>>(vpos0, vnrm0, vpos, vnrm, X);
}

void refit_read_bounds(uint32_t const *red_host, float bmin[3], float bmax[3]) {
    for (int a = 0; a < 3; a++) {
        uint32_t lo = red_host[6 + a], hi = red_host[9 + a];
        uint32_t ul = (lo & 0x80000000u) ? (lo & 0x7FFFFFFFu) : ~lo;
        uint32_t uh = (hi & 0x80000000u) ? (hi & 0x7FFFFFFFu) : ~hi;
        std::memcpy(&bmin[a], &ul, 4);
        std::memcpy(&bmax[a], &uh, 4);
    }
}

} // namespace e8g
