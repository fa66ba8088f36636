// BVH build on the device: Morton order, PLOC clustering, SAH leaf collapse, and the SAH-pair node
// layout of the host builder (bvh.h).
//
// 1. Per triangle: exact box, centroid, scene box; a 30-bit Morton code of the centroid in the
//    centroids' box; a stable LSD radix sort of (code, triangle) pairs, 8 bits per pass.
// 2. PLOC (Meister and Bittner, "Parallel Locally-Ordered Clustering for Bounding Volume
//    Hierarchy Construction", IEEE TVCG 2018): the sorted triangles are the initial clusters;
//    every round each cluster finds, among the clusters within kPlocRadius positions in the
//    current order, the one whose union box has the smallest surface area (ties to the lower
//    position); mutual nearest neighbours merge into a new node, which takes the lower position,
//    and the cluster array is compacted. The round with the globally cheapest pair always merges
//    it, so the loop ends with one cluster.
// 3. Bottom-up (a thread per triangle, the last child to arrive at a node carries on): triangle
//    counts and the SAH cost min(tri_cost A n, node_cost A + C(left) + C(right)); subtrees of at
//    most max_leaf_prims triangles whose leaf cost is not above their inner cost become leaves.
// 4. Top-down, one launch per level: every node of the level writes its 32-byte record (boxes
//    pushed out exactly as the host builder pushes them out, bvh_boxes.h) at its depth-first
//    preorder slot (the host builder's order: children adjacent, the k-th interior node's at 1 + 2k,
//    from interior-node counts of the subtrees), leaves write their triangles' records.
// Everything is deterministic: scans, not atomics, decide every position.
#include "bvh_boxes.h"
#include "gpu_build.h"
#include "launch.h"

#include <algorithm>
#include <cstring>
#include <vector>

namespace e8g {
namespace {

constexpr int kGB = 256;          // threads per block
constexpr int kSortItems = 8;     // keys per thread in the sort
constexpr int kSortTile = kGB * kSortItems;
constexpr int kScanItems = 4;     // elements per thread in the device-wide scan
constexpr int kScanTile = 1024 * kScanItems;
constexpr int kPlocRadius = 24;
constexpr int kLeafStack = 16;    // subtree walk of a leaf (at most 15 triangles)

__device__ __forceinline__ uint32_t ord_key(float f) {
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float key_float(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

// Inclusive scan of one value per thread over a block of `threads` threads (a multiple of 32).
template <int THREADS> __device__ __forceinline__ uint32_t block_inclusive(uint32_t v, uint32_t *sh) {
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t x = __shfl_up_sync(0xFFFFFFFFu, v, o);
        if (lane >= o)
            v += x;
    }
    if (lane == 31)
        sh[warp] = v;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < THREADS / 32 ? sh[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t x = __shfl_up_sync(0xFFFFFFFFu, w, o);
            if (lane >= o)
                w += x;
        }
        if (lane < THREADS / 32)
            sh[lane] = w;
    }
    __syncthreads();
    uint32_t r = v + (warp ? sh[warp - 1] : 0);
    __syncthreads();
    return r;
}

// ------------------------------------------------------------------ device-wide scan ----
// Exclusive scan in place of n values; sums[] receives one total per tile. Three launches.

__global__ void __launch_bounds__(1024) k_scan_tiles(uint32_t *d, uint32_t n, uint32_t *sums) {
    __shared__ uint32_t sh[32];
    uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    uint32_t v[kScanItems], t = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        v[k] = base + k < n ? d[base + k] : 0;
        t += v[k];
    }
    uint32_t incl = block_inclusive<1024>(t, sh);
    uint32_t run = incl - t;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        if (base + k < n)
            d[base + k] = run;
        run += v[k];
    }
    if (threadIdx.x == 1023)
        sums[blockIdx.x] = incl;
}

// Scans the tile totals (any count, one block) and writes the grand total to *total.
__global__ void __launch_bounds__(1024) k_scan_sums(uint32_t *sums, uint32_t m, uint32_t *total) {
    __shared__ uint32_t sh[32];
    uint32_t carry = 0;
    for (uint32_t b = 0; b < m; b += 1024) {
        uint32_t i = b + threadIdx.x;
        uint32_t v = i < m ? sums[i] : 0;
        uint32_t incl = block_inclusive<1024>(v, sh);
        if (i < m)
            sums[i] = carry + incl - v;
        carry += sh[31]; // the block's total
        __syncthreads();
    }
    if (threadIdx.x == 0)
        *total = carry;
}

__global__ void __launch_bounds__(1024) k_scan_add(uint32_t *d, uint32_t n, uint32_t const *sums) {
    uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    uint32_t add = sums[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; k++)
        if (base + k < n)
            d[base + k] += add;
}

// ------------------------------------------------------------------ radix sort ----

__global__ void __launch_bounds__(kGB) k_sort_hist(uint32_t const *keys, uint32_t n, int shift, uint32_t *hist) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    uint32_t base = blockIdx.x * kSortTile;
#pragma unroll
    for (int k = 0; k < kSortItems; k++) {
        uint32_t i = base + k * kGB + threadIdx.x;
        if (i < n)
            atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * gridDim.x + blockIdx.x] = h[threadIdx.x]; // digit-major
}

// Stable scatter of one tile: the tile is sorted by the digit in shared memory with eight stable
// one-bit splits, then every key goes to its digit's global offset plus its rank in the tile.
__global__ void __launch_bounds__(kGB)
    k_sort_scatter(uint32_t const *kin, uint32_t const *vin, uint32_t *kout, uint32_t *vout, uint32_t n, int shift,
                   uint32_t const *offs) {
    __shared__ uint32_t sk[kSortTile], sv[kSortTile];
    __shared__ uint32_t sh[32];
    __shared__ uint32_t start[257];
    uint32_t base = blockIdx.x * kSortTile;
    uint32_t valid = min(static_cast<uint32_t>(kSortTile), n - base);
#pragma unroll
    for (int k = 0; k < kSortItems; k++) {
        uint32_t p = k * kGB + threadIdx.x;
        sk[p] = p < valid ? kin[base + p] : 0xFFFFFFFFu; // padding sorts last and is never written
        sv[p] = p < valid ? vin[base + p] : 0u;
    }
    __syncthreads();
    uint32_t key[kSortItems], val[kSortItems];
#pragma unroll
    for (int k = 0; k < kSortItems; k++) {
        key[k] = sk[threadIdx.x * kSortItems + k];
        val[k] = sv[threadIdx.x * kSortItems + k];
    }
    __syncthreads();
    for (int b = 0; b < 8; b++) {
        int bit = shift + b;
        uint32_t zeros = 0;
#pragma unroll
        for (int k = 0; k < kSortItems; k++)
            zeros += ((key[k] >> bit) & 1u) ^ 1u;
        uint32_t incl = block_inclusive<kGB>(zeros, sh);
        uint32_t total_zeros = sh[kGB / 32 - 1]; // the block's total
        uint32_t zbefore = incl - zeros;
        uint32_t pos = threadIdx.x * kSortItems;
#pragma unroll
        for (int k = 0; k < kSortItems; k++) {
            uint32_t one = (key[k] >> bit) & 1u;
            uint32_t dst = one ? total_zeros + (pos + k - zbefore) : zbefore;
            zbefore += one ^ 1u;
            sk[dst] = key[k];
            sv[dst] = val[k];
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kSortItems; k++) {
            key[k] = sk[threadIdx.x * kSortItems + k];
            val[k] = sv[threadIdx.x * kSortItems + k];
        }
        __syncthreads();
    }
    // digit boundaries of the sorted tile
#pragma unroll
    for (int k = 0; k < kSortItems; k++) {
        uint32_t p = threadIdx.x * kSortItems + k;
        uint32_t d = (key[k] >> shift) & 255u;
        uint32_t prev = p ? (sk[p - 1] >> shift) & 255u : 0xFFFFFFFFu;
        if (p < valid && d != prev)
            start[d] = p;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kSortItems; k++) {
        uint32_t p = threadIdx.x * kSortItems + k;
        if (p < valid) {
            uint32_t d = (key[k] >> shift) & 255u;
            uint32_t dst = offs[d * gridDim.x + blockIdx.x] + (p - start[d]);
            kout[dst] = key[k];
            vout[dst] = val[k];
        }
    }
}

// ------------------------------------------------------------------ primitives ----

__global__ void k_build_init(uint32_t *red) {
    if (threadIdx.x < 12) // [0..2] min, [3..5] max of boxes; [6..8] min, [9..11] max of centroids
        red[threadIdx.x] = (threadIdx.x < 3 || (threadIdx.x >= 6 && threadIdx.x < 9)) ? 0xFFFFFFFFu : 0u;
}

template <int N, bool MAX> __device__ __forceinline__ void reduce_to(uint32_t (&v)[N], uint32_t *red) {
    __shared__ uint32_t sh[kGB / 32][N];
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
        for (int w = 1; w < kGB / 32; w++)
            r = MAX ? max(r, sh[w][threadIdx.x]) : min(r, sh[w][threadIdx.x]);
        if (MAX)
            atomicMax(&red[threadIdx.x], r);
        else
            atomicMin(&red[threadIdx.x], r);
    }
    __syncthreads();
}

// Leaf boxes (node i = triangle i before sorting) and the boxes of all boxes and of all centroids.
__global__ void __launch_bounds__(kGB) k_prim_boxes(uint4 const *tidx, float4 const *vpos, uint32_t nt, float4 *blo,
                                                     float4 *bhi, uint32_t *red) {
    uint32_t mn[6] = {~0u, ~0u, ~0u, ~0u, ~0u, ~0u}, mx[6] = {0, 0, 0, 0, 0, 0};
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += gridDim.x * blockDim.x) {
        uint4 g = tidx[t];
        float4 p0 = vpos[g.x], p1 = vpos[g.y], p2 = vpos[g.z];
        float lo[3] = {fminf(fminf(p0.x, p1.x), p2.x), fminf(fminf(p0.y, p1.y), p2.y), fminf(fminf(p0.z, p1.z), p2.z)};
        float hi[3] = {fmaxf(fmaxf(p0.x, p1.x), p2.x), fmaxf(fmaxf(p0.y, p1.y), p2.y), fmaxf(fmaxf(p0.z, p1.z), p2.z)};
        blo[t] = make_float4(lo[0], lo[1], lo[2], 0.0f);
        bhi[t] = make_float4(hi[0], hi[1], hi[2], 0.0f);
#pragma unroll
        for (int a = 0; a < 3; a++) {
            float c = 0.5f * (lo[a] + hi[a]);
            mn[a] = min(mn[a], ord_key(lo[a]));
            mx[a] = max(mx[a], ord_key(hi[a]));
            mn[3 + a] = min(mn[3 + a], ord_key(c));
            mx[3 + a] = max(mx[3 + a], ord_key(c));
        }
    }
    uint32_t a[3] = {mn[0], mn[1], mn[2]}, b[3] = {mx[0], mx[1], mx[2]};
    uint32_t c[3] = {mn[3], mn[4], mn[5]}, d[3] = {mx[3], mx[4], mx[5]};
    reduce_to<3, false>(a, red);
    reduce_to<3, true>(b, red + 3);
    reduce_to<3, false>(c, red + 6);
    reduce_to<3, true>(d, red + 9);
}

__device__ __forceinline__ uint32_t spread10(uint32_t v) {
    v &= 0x3FFu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

__global__ void k_morton(float4 const *blo, float4 const *bhi, uint32_t nt, uint32_t const *red, uint32_t *keys,
                         uint32_t *vals) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt)
        return;
    float4 lo = blo[t], hi = bhi[t];
    float c[3] = {0.5f * (lo.x + hi.x), 0.5f * (lo.y + hi.y), 0.5f * (lo.z + hi.z)};
    uint32_t code = 0;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        float cl = key_float(red[6 + a]), ch = key_float(red[9 + a]);
        float ext = ch - cl;
        float u = ext > 0.0f ? (c[a] - cl) / ext : 0.0f;
        uint32_t q = static_cast<uint32_t>(fminf(fmaxf(u * 1024.0f, 0.0f), 1023.0f));
        code |= spread10(q) << (2 - a);
    }
    keys[t] = code;
    vals[t] = t;
}

// Leaf nodes 0..n-1 in sorted order: boxes gathered from the triangle boxes.
__global__ void k_gather_leaves(uint32_t const *order, float4 const *tlo, float4 const *thi, uint32_t n, float4 *blo,
                                float4 *bhi, uint32_t *clusters) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    uint32_t t = order[i];
    blo[i] = tlo[t];
    bhi[i] = thi[t];
    clusters[i] = i;
}

// ------------------------------------------------------------------------ PLOC ----

__device__ __forceinline__ float union_area(float4 a0, float4 a1, float4 b0, float4 b1) {
    float dx = fmaxf(a1.x, b1.x) - fminf(a0.x, b0.x);
    float dy = fmaxf(a1.y, b1.y) - fminf(a0.y, b0.y);
    float dz = fmaxf(a1.z, b1.z) - fminf(a0.z, b0.z);
    return dx * dy + dy * dz + dz * dx;
}

__global__ void __launch_bounds__(kGB) k_ploc_nn(uint32_t const *clus, uint32_t m, float4 const *blo,
                                                  float4 const *bhi, int32_t *nn) {
    __shared__ float4 slo[kGB + 2 * kPlocRadius], shi[kGB + 2 * kPlocRadius];
    int s0 = static_cast<int>(blockIdx.x * kGB) - kPlocRadius;
    for (int k = threadIdx.x; k < kGB + 2 * kPlocRadius; k += kGB) {
        int idx = s0 + k;
        if (idx >= 0 && idx < static_cast<int>(m)) {
            uint32_t node = clus[idx];
            slo[k] = blo[node];
            shi[k] = bhi[node];
        }
    }
    __syncthreads();
    int i = static_cast<int>(blockIdx.x * kGB + threadIdx.x);
    if (i >= static_cast<int>(m))
        return;
    float4 a0 = slo[threadIdx.x + kPlocRadius], a1 = shi[threadIdx.x + kPlocRadius];
    float best = INFINITY;
    int bj = -1;
    for (int d = -kPlocRadius; d <= kPlocRadius; d++) {
        int j = i + d;
        if (d == 0 || j < 0 || j >= static_cast<int>(m))
            continue;
        float area = union_area(a0, a1, slo[threadIdx.x + kPlocRadius + d], shi[threadIdx.x + kPlocRadius + d]);
        if (area < best) { // increasing j: ties keep the lower position
            best = area;
            bj = j;
        }
    }
    nn[i] = bj;
}

__global__ void k_ploc_flags(int32_t const *nn, uint32_t m, uint32_t *merged, uint32_t *keep) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m)
        return;
    int32_t j = nn[i];
    bool mutual = j >= 0 && nn[j] == static_cast<int32_t>(i);
    merged[i] = mutual && static_cast<int32_t>(i) < j;
    keep[i] = !(mutual && static_cast<int32_t>(i) > j);
}

__global__ void k_ploc_apply(uint32_t const *clus, uint32_t *clus_out, int32_t const *nn, uint32_t m,
                             uint32_t const *mscan, uint32_t const *kscan, uint32_t const *mflag,
                             uint32_t const *kflag, uint32_t base, float4 *blo, float4 *bhi, int2 *child) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m || !kflag[i])
        return;
    if (mflag[i]) {
        uint32_t node = base + mscan[i]; // < 2n - 1: every merge removes one cluster
        uint32_t a = clus[i], b = clus[nn[i]];
        child[node] = make_int2(static_cast<int>(a), static_cast<int>(b));
        float4 a0 = blo[a], a1 = bhi[a], b0 = blo[b], b1 = bhi[b];
        blo[node] = make_float4(fminf(a0.x, b0.x), fminf(a0.y, b0.y), fminf(a0.z, b0.z), 0.0f);
        bhi[node] = make_float4(fmaxf(a1.x, b1.x), fmaxf(a1.y, b1.y), fmaxf(a1.z, b1.z), 0.0f);
        clus_out[kscan[i]] = node;
    } else {
        clus_out[kscan[i]] = clus[i];
    }
}

// The last rounds, once few clusters are left, in one block: the same rounds as the kernels above
// (same neighbour search, tie-breaks and node numbering), without a launch and a host read per
// round.
constexpr int kPlocSmall = 2048;  // clusters the one-block kernel takes over at
constexpr int kPlocSmallThreads = 1024;

__global__ void __launch_bounds__(kPlocSmallThreads)
    k_ploc_finish(uint32_t const *clus_in, uint32_t m, uint32_t base, float4 *blo, float4 *bhi, int2 *child,
                  uint32_t *out_nodes) {
    __shared__ uint32_t ca[kPlocSmall], cb[kPlocSmall];
    __shared__ int32_t nn[kPlocSmall];
    __shared__ uint32_t ms[kPlocSmall], ks[kPlocSmall];
    __shared__ uint32_t sh[32];
    constexpr int per = kPlocSmall / kPlocSmallThreads; // elements per thread in the scans
    for (uint32_t i = threadIdx.x; i < m; i += kPlocSmallThreads)
        ca[i] = clus_in[i];
    __syncthreads();
    uint32_t *cur = ca, *nxt = cb;
    int rounds = 0;
    while (m > 1 && rounds++ < 1000000) {
        for (uint32_t i = threadIdx.x; i < m; i += kPlocSmallThreads) {
            uint32_t node = cur[i];
            float4 a0 = blo[node], a1 = bhi[node];
            float best = INFINITY;
            int bj = -1;
            for (int d = -kPlocRadius; d <= kPlocRadius; d++) {
                int j = static_cast<int>(i) + d;
                if (d == 0 || j < 0 || j >= static_cast<int>(m))
                    continue;
                uint32_t o = cur[j];
                float area = union_area(a0, a1, blo[o], bhi[o]);
                if (area < best) {
                    best = area;
                    bj = j;
                }
            }
            nn[i] = bj;
        }
        __syncthreads();
        // merge flags and their exclusive scans (each thread owns `per` consecutive clusters)
        uint32_t mf[per], kf[per], msum = 0, ksum = 0;
#pragma unroll
        for (int k = 0; k < per; k++) {
            uint32_t i = threadIdx.x * per + k;
            uint32_t merged = 0, keep = 0;
            if (i < m) {
                int32_t j = nn[i];
                bool mutual = j >= 0 && nn[j] == static_cast<int32_t>(i);
                merged = mutual && static_cast<int32_t>(i) < j;
                keep = !(mutual && static_cast<int32_t>(i) > j);
            }
            mf[k] = merged;
            kf[k] = keep;
            msum += merged;
            ksum += keep;
        }
        uint32_t mincl = block_inclusive<kPlocSmallThreads>(msum, sh);
        uint32_t mtotal = sh[31];
        __syncthreads();
        uint32_t kincl = block_inclusive<kPlocSmallThreads>(ksum, sh);
        uint32_t ktotal = sh[31];
        __syncthreads();
        uint32_t mrun = mincl - msum, krun = kincl - ksum;
#pragma unroll
        for (int k = 0; k < per; k++) {
            uint32_t i = threadIdx.x * per + k;
            if (i < m) {
                ms[i] = mf[k] ? mrun : 0xFFFFFFFFu;
                ks[i] = kf[k] ? krun : 0xFFFFFFFFu;
            }
            mrun += mf[k];
            krun += kf[k];
        }
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < m; i += kPlocSmallThreads) {
            if (ks[i] == 0xFFFFFFFFu)
                continue;
            if (ms[i] != 0xFFFFFFFFu) {
                uint32_t node = base + ms[i];
                uint32_t a = cur[i], b = cur[nn[i]];
                child[node] = make_int2(static_cast<int>(a), static_cast<int>(b));
                float4 a0 = blo[a], a1 = bhi[a], b0 = blo[b], b1 = bhi[b];
                blo[node] = make_float4(fminf(a0.x, b0.x), fminf(a0.y, b0.y), fminf(a0.z, b0.z), 0.0f);
                bhi[node] = make_float4(fmaxf(a1.x, b1.x), fmaxf(a1.y, b1.y), fmaxf(a1.z, b1.z), 0.0f);
                nxt[ks[i]] = node;
            } else {
                nxt[ks[i]] = cur[i];
            }
        }
        __syncthreads();
        if (mtotal == 0)
            break; // no mutual pair (non-finite boxes): reported through the node count
        base += mtotal;
        m = ktotal;
        uint32_t *t = cur;
        cur = nxt;
        nxt = t;
        __threadfence_block();
        __syncthreads();
    }
    if (threadIdx.x == 0)
        out_nodes[0] = m == 1 ? base : 0u;
}

// ------------------------------------------------------------- collapse (bottom-up) ----

__global__ void k_tree_parents(int2 const *child, uint32_t n, uint32_t num_nodes, uint32_t *parent) {
    uint32_t node = n + blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= num_nodes)
        return;
    int2 c = child[node];
    parent[c.x] = node;
    parent[c.y] = node;
}

__device__ __forceinline__ float box_area(float4 lo, float4 hi) {
    float dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
    return dx * dy + dy * dz + dz * dx;
}

// Triangle counts, SAH cost and leaf decisions; a thread per triangle walks up.
__global__ void k_collapse(uint32_t n, int2 const *child, uint32_t const *parent, float4 const *blo,
                           float4 const *bhi, uint32_t *counter, uint32_t *ntris, uint32_t *icount, float *cost,
                           uint8_t *leaf, uint32_t max_leaf, float tri_cost, float node_cost) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    ntris[i] = 1;
    icount[i] = 0;
    cost[i] = tri_cost * box_area(blo[i], bhi[i]);
    leaf[i] = 1;
    uint32_t node = parent[i];
    while (node != 0xFFFFFFFFu) {
        // the second child to arrive carries on: release of this thread's writes, acquire of the
        // sibling's
        uint32_t old;
        asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;" : "=r"(old) : "l"(&counter[node]) : "memory");
        if (old == 0)
            return;
        int2 c = child[node];
        uint32_t cnt = __ldcg(&ntris[c.x]) + __ldcg(&ntris[c.y]);
        float area = box_area(blo[node], bhi[node]);
        float inner = node_cost * area + __ldcg(&cost[c.x]) + __ldcg(&cost[c.y]);
        float as_leaf = tri_cost * area * static_cast<float>(cnt);
        bool make_leaf = cnt <= max_leaf && as_leaf <= inner;
        ntris[node] = cnt;
        icount[node] = make_leaf ? 0u : 1u + __ldcg(&icount[c.x]) + __ldcg(&icount[c.y]);
        cost[node] = make_leaf ? as_leaf : inner;
        leaf[node] = make_leaf;
        node = parent[node];
    }
}

// ------------------------------------------------------------ flatten (top-down) ----

struct FlatItem {
    uint32_t node, slot, tri_start;
    uint32_t pre; // interior nodes before this one in depth-first preorder
};

struct WideItem {
    uint32_t bn, wn; // binary node, wide node index
};

__global__ void k_flat_flags(FlatItem const *items, uint32_t f, uint8_t const *leaf, uint32_t *interior) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < f)
        interior[i] = leaf[items[i].node] ? 0u : 1u;
}

__global__ void k_flat_emit(FlatItem const *items, uint32_t f, uint32_t const *iscan, uint32_t n, int2 const *child,
                            uint8_t const *leaf, uint32_t const *ntris, uint32_t const *icount, float4 const *blo,
                            float4 const *bhi, uint32_t const *order, uint4 const *tidx, float4 const *vpos,
                            uint32_t const *red, float4 *nlo, float4 *nhi, float4 *tri, FlatItem *next,
                            unsigned long long *leaf_stats) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= f)
        return;
    FlatItem it = items[i];
    float lo[3], hi[3];
    for (int a = 0; a < 3; a++) {
        lo[a] = key_float(red[a]);
        hi[a] = key_float(red[3 + a]);
    }
    float eps = scene_eps(lo, hi);
    float4 b0 = blo[it.node], b1 = bhi[it.node];
    uint32_t link, count;
    if (leaf[it.node]) {
        link = it.tri_start;
        count = ntris[it.node];
        // the leaf's triangles, left to right
        uint32_t stack[kLeafStack];
        int sp = 0, k = 0;
        stack[sp++] = it.node;
        while (sp > 0) {
            uint32_t x = stack[--sp];
            if (x < n) {
                uint32_t t = order[x];
                uint4 g = tidx[t];
                float4 p0 = vpos[g.x], p1 = vpos[g.y], p2 = vpos[g.z];
                size_t r = 3 * static_cast<size_t>(it.tri_start + k);
                tri[r] = make_float4(p0.x, p0.y, p0.z, __uint_as_float(t));
                tri[r + 1] = make_float4(p1.x - p0.x, p1.y - p0.y, p1.z - p0.z, 0.0f);
                tri[r + 2] = make_float4(p2.x - p0.x, p2.y - p0.y, p2.z - p0.z, 0.0f);
                k++;
            } else if (sp + 2 <= kLeafStack) {
                int2 c = child[x];
                stack[sp++] = static_cast<uint32_t>(c.y);
                stack[sp++] = static_cast<uint32_t>(c.x);
            }
        }
        atomicAdd(&leaf_stats[0], 1ull);
    } else {
        // depth-first preorder slots, as the host builder lays nodes out: the k-th interior node in
        // preorder keeps its children at 1 + 2k and 2 + 2k
        link = 1 + 2 * it.pre;
        count = 0;
        int2 c = child[it.node];
        next[2 * iscan[i]] = FlatItem{static_cast<uint32_t>(c.x), link, it.tri_start, it.pre + 1};
        next[2 * iscan[i] + 1] =
            FlatItem{static_cast<uint32_t>(c.y), link + 1, it.tri_start + ntris[c.x], it.pre + 1 + icount[c.x]};
    }
    nlo[it.slot] = make_float4(inflate_lo(b0.x, eps), inflate_lo(b0.y, eps), inflate_lo(b0.z, eps),
                               __uint_as_float(link));
    nhi[it.slot] = make_float4(inflate_hi(b1.x, eps), inflate_hi(b1.y, eps), inflate_hi(b1.z, eps),
                               __uint_as_float(count));
}

inline uint32_t blocks(uint64_t n, int per) { return n ? static_cast<uint32_t>((n + per - 1) / per) : 1u; }

struct Carver {
    char *p;
    size_t used = 0;
    template <class T> T *take(size_t count) {
        size_t off = (used + 255) & ~size_t(255);
        used = off + count * sizeof(T);
        return p ? reinterpret_cast<T *>(p + off) : nullptr;
    }
};

struct Scratch {
    uint32_t *red, *keys0, *vals0, *keys1, *vals1, *hist, *sums, *total;
    float4 *tlo, *thi, *blo, *bhi;
    int2 *child;
    uint32_t *clus0, *clus1, *mflag, *kflag, *mscan, *kscan, *parent, *counter, *ntris, *icount;
    int32_t *nn;
    float *cost;
    uint8_t *leaf;
    FlatItem *fa, *fb;
    uint32_t *iflag;
    unsigned long long *leaf_stats;
    WideItem *wa, *wb;   // eight-wide collapse: frontiers,
    uint32_t *wslots;    // 8 chosen children per frontier node,
    float4 *tri_tmp;     // triangle records in the wide order
};

Scratch carve(void *base, uint32_t n, size_t *bytes) {
    Carver c{static_cast<char *>(base)};
    Scratch s;
    size_t nodes = 2 * static_cast<size_t>(n);
    uint32_t sort_blocks = blocks(n, kSortTile);
    size_t hist_n = 256 * static_cast<size_t>(sort_blocks);
    size_t scan_max = std::max<size_t>(hist_n, n);
    s.red = c.take<uint32_t>(16);
    s.total = c.take<uint32_t>(4);
    s.keys0 = c.take<uint32_t>(n);
    s.vals0 = c.take<uint32_t>(n);
    s.keys1 = c.take<uint32_t>(n);
    s.vals1 = c.take<uint32_t>(n);
    s.hist = c.take<uint32_t>(hist_n);
    s.sums = c.take<uint32_t>(blocks(scan_max, kScanTile) + 1);
    s.tlo = c.take<float4>(n);
    s.thi = c.take<float4>(n);
    s.blo = c.take<float4>(nodes);
    s.bhi = c.take<float4>(nodes);
    s.child = c.take<int2>(nodes);
    s.clus0 = c.take<uint32_t>(n);
    s.clus1 = c.take<uint32_t>(n);
    s.mflag = c.take<uint32_t>(n);
    s.kflag = c.take<uint32_t>(n);
    s.mscan = c.take<uint32_t>(n);
    s.kscan = c.take<uint32_t>(n);
    s.nn = c.take<int32_t>(n);
    s.parent = c.take<uint32_t>(nodes);
    s.counter = c.take<uint32_t>(nodes);
    s.ntris = c.take<uint32_t>(nodes);
    s.icount = c.take<uint32_t>(nodes);
    s.cost = c.take<float>(nodes);
    s.leaf = c.take<uint8_t>(nodes);
    s.fa = c.take<FlatItem>(nodes);
    s.fb = c.take<FlatItem>(nodes);
    s.iflag = c.take<uint32_t>(nodes);
    s.leaf_stats = c.take<unsigned long long>(2);
    s.wa = c.take<WideItem>(n);
    s.wb = c.take<WideItem>(n);
    s.wslots = c.take<uint32_t>(8 * static_cast<size_t>(n));
    s.tri_tmp = c.take<float4>(3 * static_cast<size_t>(n));
    *bytes = c.used + 256;
    return s;
}

// Exclusive scan of d[0, n) in place; the total lands in *total (device).
void scan(uint32_t *d, uint32_t n, uint32_t *sums, uint32_t *total, cudaStream_t st) {
    uint32_t tiles = blocks(n, kScanTile);
    k_scan_tiles<<<tiles, 1024, 0, st>>>(d, n, sums);
    k_scan_sums<<<1, 1024, 0, st>>>(sums, tiles, total);
    k_scan_add<<<tiles, 1024, 0, st>>>(d, n, sums);
}

// ------------------------------------------------------------ eight-wide collapse ----
// The host collapse (bvh_wide.cpp) level by level: a thread per wide node opens the binary child
// with the largest surface area until eight children are collected, assigns octant slots with the
// same greedy cost and quantizes with the same arithmetic; scans give every node the child and
// triangle bases the host's breadth-first queue gives it, so the bytes equal the host's.

__device__ __forceinline__ float wide_area(float4 lo, float4 hi) {
    float d0 = hi.x - lo.x, d1 = hi.y - lo.y, d2 = hi.z - lo.z;
    if (!(d0 >= 0) || !(d1 >= 0) || !(d2 >= 0))
        return 0.0f;
    return 2.0f * (d0 * d1 + d0 * d2 + d1 * d2);
}

// Children of one wide node in slot order (binary node ids, kNone for an empty slot).
constexpr uint32_t kNone = 0xFFFFFFFFu;

__device__ void wide_children(uint32_t bn, float4 const *nlo, float4 const *nhi, uint32_t slots[8]) {
    uint32_t ch[8];
    int n = 0;
    if (__float_as_uint(nhi[bn].w) == 0) {
        uint32_t l = __float_as_uint(nlo[bn].w);
        ch[0] = l;
        ch[1] = l + 1;
        n = 2;
        while (n < 8) {
            int best = -1;
            float best_area = -1.0f;
            for (int i = 0; i < n; i++)
                if (__float_as_uint(nhi[ch[i]].w) == 0) {
                    float a = wide_area(nlo[ch[i]], nhi[ch[i]]);
                    if (a > best_area) {
                        best = i;
                        best_area = a;
                    }
                }
            if (best < 0)
                break;
            uint32_t l = __float_as_uint(nlo[ch[best]].w);
            ch[best] = l;
            ch[n++] = l + 1;
        }
    } else {
        ch[0] = bn; // a root that is a leaf
        n = 1;
    }
    float ulo[3] = {INFINITY, INFINITY, INFINITY}, uhi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int i = 0; i < n; i++) {
        float4 a = nlo[ch[i]], b = nhi[ch[i]];
        ulo[0] = a.x < ulo[0] ? a.x : ulo[0];
        ulo[1] = a.y < ulo[1] ? a.y : ulo[1];
        ulo[2] = a.z < ulo[2] ? a.z : ulo[2];
        uhi[0] = uhi[0] < b.x ? b.x : uhi[0];
        uhi[1] = uhi[1] < b.y ? b.y : uhi[1];
        uhi[2] = uhi[2] < b.z ? b.z : uhi[2];
    }
    float cost[8][8];
    for (int i = 0; i < n; i++) {
        float4 a = nlo[ch[i]], b = nhi[ch[i]];
        float lo[3] = {a.x, a.y, a.z}, hi[3] = {b.x, b.y, b.z};
        for (int s = 0; s < 8; s++) {
            float c = 0;
            for (int ax = 0; ax < 3; ax++) {
                float off = 0.5f * (lo[ax] + hi[ax]) - 0.5f * (ulo[ax] + uhi[ax]);
                c += (s >> ax & 1) ? -off : off;
            }
            cost[i][s] = c;
        }
    }
    int slot_of[8], child_in[8];
    for (int i = 0; i < 8; i++)
        slot_of[i] = child_in[i] = -1;
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
    for (int s = 0; s < 8; s++)
        slots[s] = child_in[s] < 0 ? kNone : ch[child_in[s]];
}

__global__ void k_wide_plan(WideItem const *items, uint32_t f, float4 const *nlo, float4 const *nhi,
                            uint32_t *slots_out, uint32_t *n_int, uint32_t *n_tri) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= f)
        return;
    uint32_t slots[8];
    wide_children(items[i].bn, nlo, nhi, slots);
    uint32_t ni = 0, nt = 0;
    for (int s = 0; s < 8; s++) {
        slots_out[8 * static_cast<size_t>(i) + s] = slots[s];
        if (slots[s] == kNone)
            continue;
        uint32_t cnt = __float_as_uint(nhi[slots[s]].w);
        if (cnt == 0)
            ni++;
        else
            nt += cnt;
    }
    n_int[i] = ni;
    n_tri[i] = nt;
}

__global__ void k_wide_emit(WideItem const *items, uint32_t f, uint32_t const *slots_in, uint32_t const *int_scan,
                            uint32_t const *tri_scan, uint32_t next_base, uint32_t tri_running, float4 const *nlo,
                            float4 const *nhi, float4 const *tri_bin, float4 *tri_wide, double step_min, uint4 *wide,
                            WideItem *next) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= f)
        return;
    uint32_t words[24];
    for (int k = 0; k < 24; k++)
        words[k] = 0;
    float slo[8][3], shi[8][3];
    uint32_t present = 0, imask = 0, leaves = 0, counts = 0;
    uint32_t child_base = next_base + int_scan[i], tri_base = tri_running + tri_scan[i];
    uint32_t rank = 0, toff = 0;
    uint32_t meta[2] = {0, 0};
    for (int s = 0; s < 8; s++) {
        uint32_t c = slots_in[8 * static_cast<size_t>(i) + s];
        if (c == kNone) {
            for (int a = 0; a < 3; a++)
                slo[s][a] = shi[s][a] = 0.0f;
            continue;
        }
        float4 a = nlo[c], b = nhi[c];
        slo[s][0] = a.x, slo[s][1] = a.y, slo[s][2] = a.z;
        shi[s][0] = b.x, shi[s][1] = b.y, shi[s][2] = b.z;
        present |= 1u << s;
        uint32_t cnt = __float_as_uint(b.w);
        if (cnt == 0) {
            imask |= 1u << s;
            next[int_scan[i] + rank] = WideItem{c, child_base + rank};
            rank++;
        } else {
            meta[s >> 2] |= toff << (8 * (s & 3));
            counts |= cnt << (4 * s);
            leaves |= 1u << s;
            uint32_t first = __float_as_uint(a.w);
            for (uint32_t k = 0; k < cnt; k++) {
                size_t src = 3 * static_cast<size_t>(first + k), dst = 3 * static_cast<size_t>(tri_base + toff + k);
                tri_wide[dst] = tri_bin[src];
                tri_wide[dst + 1] = tri_bin[src + 1];
                tri_wide[dst + 2] = tri_bin[src + 2];
            }
            toff += cnt;
        }
    }
    wide_quantize(slo, shi, present, step_min, words);
    words[3] |= imask << 24;
    words[4] = child_base;
    words[5] = tri_base;
    words[6] = meta[0];
    words[7] = meta[1];
    words[20] = counts;
    words[21] = leaves;
    uint4 *dst = wide + 6 * static_cast<size_t>(items[i].wn);
    for (int q = 0; q < 6; q++)
        dst[q] = make_uint4(words[4 * q], words[4 * q + 1], words[4 * q + 2], words[4 * q + 3]);
}

} // namespace

size_t gpu_build_scratch_bytes(uint32_t num_tris) {
    size_t bytes = 0;
    carve(nullptr, num_tris, &bytes);
    return bytes;
}

cudaError_t gpu_build_sah_pairs(GpuBuildIn const &in, GpuBuildOut &out, cudaStream_t st) {
    uint32_t n = in.num_tris;
    out = GpuBuildOut{};
    if (n == 0)
        return cudaSuccess;
    size_t bytes = 0;
    Scratch s = carve(in.scratch, n, &bytes);
    uint32_t *host = static_cast<uint32_t *>(in.host_pinned); // 4 words of pinned host memory
    int grid_cap = 8 * in.num_sms;
    // 1. boxes, Morton codes, sort
    k_build_init<<<1, 32, 0, st>>>(s.red);
    k_prim_boxes<<<std::min<uint32_t>(blocks(n, kGB), grid_cap), kGB, 0, st>>>(in.tidx, in.vpos, n, s.tlo, s.thi, s.red);
    k_morton<<<blocks(n, kGB), kGB, 0, st>>>(s.tlo, s.thi, n, s.red, s.keys0, s.vals0);
    uint32_t sort_blocks = blocks(n, kSortTile);
    uint32_t *kin = s.keys0, *vin = s.vals0, *kout = s.keys1, *vout = s.vals1;
    for (int shift = 0; shift < 32; shift += 8) {
        k_sort_hist<<<sort_blocks, kGB, 0, st>>>(kin, n, shift, s.hist);
        scan(s.hist, 256 * sort_blocks, s.sums, s.total, st);
        k_sort_scatter<<<sort_blocks, kGB, 0, st>>>(kin, vin, kout, vout, n, shift, s.hist);
        std::swap(kin, kout);
        std::swap(vin, vout);
    }
    uint32_t *order = vin; // sorted position -> triangle
    k_gather_leaves<<<blocks(n, kGB), kGB, 0, st>>>(order, s.tlo, s.thi, n, s.blo, s.bhi, s.clus0);
    // 2. PLOC rounds
    uint32_t m = n, base = n;
    uint32_t *ca = s.clus0, *cb = s.clus1;
    int rounds = 0;
    while (m > 1) {
        if (m <= static_cast<uint32_t>(kPlocSmall)) {
            // the remaining rounds in one block
            k_ploc_finish<<<1, kPlocSmallThreads, 0, st>>>(ca, m, base, s.blo, s.bhi, s.child, s.total + 2);
            cudaError_t e = cudaMemcpyAsync(host, s.total + 2, 4, cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess)
                e = cudaStreamSynchronize(st);
            if (e != cudaSuccess)
                return e;
            if (host[0] == 0)
                return cudaErrorUnknown; // no mutual pair (non-finite boxes): host build
            base = host[0];
            m = 1;
            break;
        }
        if (++rounds > 100000)
            return cudaErrorUnknown; // no progress: the caller falls back to the host build
        uint32_t g = blocks(m, kGB);
        k_ploc_nn<<<g, kGB, 0, st>>>(ca, m, s.blo, s.bhi, s.nn);
        k_ploc_flags<<<g, kGB, 0, st>>>(s.nn, m, s.mflag, s.kflag);
        cudaMemcpyAsync(s.mscan, s.mflag, 4 * static_cast<size_t>(m), cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(s.kscan, s.kflag, 4 * static_cast<size_t>(m), cudaMemcpyDeviceToDevice, st);
        scan(s.mscan, m, s.sums, s.total, st);
        scan(s.kscan, m, s.sums, s.total + 1, st);
        k_ploc_apply<<<g, kGB, 0, st>>>(ca, cb, s.nn, m, s.mscan, s.kscan, s.mflag, s.kflag, base, s.blo, s.bhi,
                                        s.child);
        cudaMemcpyAsync(host, s.total, 8, cudaMemcpyDeviceToHost, st);
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess)
            return e;
        if (host[0] == 0)
            return cudaErrorUnknown; // no mutual pair (non-finite boxes): host build
        base += host[0];
        m = host[1];
        std::swap(ca, cb);
    }
    uint32_t num_nodes = base, root = num_nodes - 1;
    // 3. leaf collapse
    cudaMemsetAsync(s.parent, 0xFF, 4 * static_cast<size_t>(num_nodes), st);
    if (num_nodes > n)
        k_tree_parents<<<blocks(num_nodes - n, kGB), kGB, 0, st>>>(s.child, n, num_nodes, s.parent);
    cudaMemsetAsync(s.counter, 0, 4 * static_cast<size_t>(num_nodes), st);
    k_collapse<<<blocks(n, kGB), kGB, 0, st>>>(n, s.child, s.parent, s.blo, s.bhi, s.counter, s.ntris, s.icount, s.cost,
                                               s.leaf, in.max_leaf, in.tri_cost, in.node_cost);
    // 4. flatten level by level
    FlatItem first{root, 0, 0, 0};
    cudaMemcpyAsync(s.fa, &first, sizeof(first), cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(s.leaf_stats, 0, 16, st);
    uint32_t f = 1, slot_base = 1, depth = 0;
    uint64_t leaf_depth_sum = 0;
    FlatItem *fa = s.fa, *fb = s.fb;
    while (f > 0) {
        depth++;
        // a level never holds more nodes than there are triangles; anything else is a malformed
        // tree, which is refused before a write could leave the buffers
        if (f > n || slot_base > 2ull * n)
            return cudaErrorUnknown;
        if (depth > in.max_depth) { // deeper than the traversal stack: the host builds instead
            out.ok = false;
            return cudaSuccess;
        }
        uint32_t g = blocks(f, kGB);
        k_flat_flags<<<g, kGB, 0, st>>>(fa, f, s.leaf, s.iflag);
        scan(s.iflag, f, s.sums, s.total, st);
        k_flat_emit<<<g, kGB, 0, st>>>(fa, f, s.iflag, n, s.child, s.leaf, s.ntris, s.icount, s.blo, s.bhi, order,
                                       in.tidx, in.vpos, s.red, in.nlo, in.nhi, in.tri, fb, s.leaf_stats);
        cudaMemcpyAsync(host, s.total, 4, cudaMemcpyDeviceToHost, st);
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess)
            return e;
        uint32_t interior = host[0];
        leaf_depth_sum += static_cast<uint64_t>(f - interior) * (depth - 1);
        slot_base += 2 * interior;
        f = 2 * interior;
        std::swap(fa, fb);
    }
    out.num_nodes = slot_base;
    unsigned long long leaves = 0;
    cudaError_t e = cudaMemcpyAsync(host, s.leaf_stats, 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(host + 2, s.red, 24, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
        return e;
    std::memcpy(&leaves, host, 8);
    for (int a = 0; a < 3; a++) {
        uint32_t lo = host[2 + a], hi = host[5 + a];
        uint32_t ul = (lo & 0x80000000u) ? (lo & 0x7FFFFFFFu) : ~lo;
        uint32_t uh = (hi & 0x80000000u) ? (hi & 0x7FFFFFFFu) : ~hi;
        std::memcpy(&out.scene_lo[a], &ul, 4);
        std::memcpy(&out.scene_hi[a], &uh, 4);
    }
    out.num_leaves = static_cast<uint32_t>(leaves);
    out.max_depth = depth;
    out.avg_leaf_depth = leaves ? static_cast<double>(leaf_depth_sum) / static_cast<double>(leaves) : 0.0;
    out.ploc_rounds = static_cast<uint32_t>(rounds);
    out.ok = depth <= in.max_depth;
    return cudaGetLastError();
}

} // namespace e8g

namespace e8g {

cudaError_t gpu_collapse_wide(GpuWideIn const &in, GpuWideOut &out, cudaStream_t st) {
    uint32_t n = in.num_tris;
    out = GpuWideOut{};
    if (n == 0)
        return cudaSuccess;
    size_t bytes = 0;
    Scratch s = carve(in.scratch, n, &bytes);
    uint32_t *host = static_cast<uint32_t *>(in.host_pinned);
    double step_min = wide_step_min(in.max_abs);
    WideItem root{0, 0};
    cudaError_t e = cudaMemcpyAsync(s.wa, &root, sizeof(root), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess)
        return e;
    uint32_t f = 1, next_base = 1, tri_running = 0, depth = 0, level_first = 0;
    WideItem *wa = s.wa, *wb = s.wb;
    while (f > 0) {
        if (++depth > in.max_depth || depth >= 32 || f > n || next_base > n + 1) {
            out.ok = false; // too deep for the eight-wide stack: keep the binary tree
            return cudaSuccess;
        }
        out.level_start[depth - 1] = level_first; // this level's nodes are [level_first, next_base)
        level_first = next_base;
        uint32_t g = blocks(f, kGB);
        k_wide_plan<<<g, kGB, 0, st>>>(wa, f, in.nlo, in.nhi, s.wslots, s.mscan, s.kscan);
        scan(s.mscan, f, s.sums, s.total, st);
        scan(s.kscan, f, s.sums, s.total + 1, st);
        k_wide_emit<<<g, kGB, 0, st>>>(wa, f, s.wslots, s.mscan, s.kscan, next_base, tri_running, in.nlo, in.nhi,
                                       in.tri, s.tri_tmp, step_min, in.wide, wb);
        e = cudaMemcpyAsync(host, s.total, 8, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(st);
        if (e != cudaSuccess)
            return e;
        next_base += host[0];
        tri_running += host[1];
        f = host[0];
        std::swap(wa, wb);
    }
    if (tri_running != n)
        return cudaErrorUnknown;
    // the triangle records move to the wide order only now that the collapse succeeded
    e = cudaMemcpyAsync(in.tri, s.tri_tmp, 48 * static_cast<size_t>(n), cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess)
        return e;
    out.num_nodes = next_base;
    out.max_depth = depth;
    out.level_start[depth] = next_base;
    out.ok = true;
    return cudaGetLastError();
}

} // namespace e8g
