// SAH binned BVH build on the GPU: BvhBuilder::build_for (BT/src/model/bvh.rs:317-541) with the
// same node array, triangle order and permutation as the host build, bit for bit.
//
// The reference recurses depth-first and partitions each node with a sequential swap loop.  Here
// the nodes of one tree level are processed together, and every per-triangle step runs in tiles
// of up to 2,048 triangles of one node (one block per tile: block reductions, then one atomic per
// node and quantity):
//  1. node bounds (update_node_bounds, bvh.rs:317-330) and centroid bounds per axis
//     (find_best_split_plane, bvh.rs:333-352): the reference's f32::min / f32::max folds, reduced
//     with 64-bit keys (value rank, position in the fold's order) so that the first of equal
//     values wins as in the fold; the fold's starting value wins where no element beats it;
//  2. the 8 bins per axis (bvh.rs:354-366): counts, and bin boxes grown from the zero box;
//  3. per node, one thread: the sweep, costs and split choice (bvh.rs:368-394) and the no-split
//     test (bvh.rs:398-417) in the reference's operation order;
//  4. the partition (bvh.rs:419-435) as a scatter.  With L triangles going left, the swap loop
//     leaves every left triangle of [first, first+L) in place; the k-th left triangle of
//     [first+L, end), counted from the end (l_k), takes the place of the k-th right triangle of
//     [first, first+L) (r_k); r_1 goes to the last position and r_k (k > 1) just below l_(k-1);
//     every other right triangle of [first+L, end) moves down by one, except the one at first+L,
//     which goes just below l_m (to the last position when m = 0).  This closed form was checked
//     against the sequential loop on random inputs; it also covers the reference's rotation of a
//     node whose triangles all go right (first > 0: the split is then abandoned, the order kept).
//  5. the children of split nodes form the next level.
// The reference numbers nodes as its recursion splits them (left subtree first): node 0 is the
// root, node 1 unused, and the children of the s-th split node in depth-first pre-order are
// 2 + 2s and 3 + 2s.  That numbering is assigned on the host from the level topology at the end.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "internal.hpp"

namespace bvhgpu {
namespace {

constexpr int kThreads = 256;
constexpr uint32_t kTile = 2048;  // triangles per tile; 8 per thread
constexpr uint32_t kPerThread = kTile / kThreads;
constexpr unsigned long long kMinId = 0xFFFFFFFFFFFFFFFFull;
constexpr unsigned long long kMaxId = 0ull;
// keys per node: node bounds (3 min + 3 max), centroid bounds (3 + 3), bins (3 axes x 8 bins x
// 3 components, min and max)
constexpr int kKeysNb = 0, kKeysCb = 3, kKeysBin = 6, kKeysPerNode = 6 + 72;

struct Tile {
    uint32_t node, begin, end, pad;
};

struct LevelNode {
    uint32_t first, count, tile_begin, tile_end;
    float lo[3], hi[3];
    float cmin[3], cmax[3], scale[3];
    uint32_t active;   // bit k: axis k is binned (its centroid bounds differ)
    uint32_t attempt;  // the SAH cost beats the leaf cost: the partition runs
    int32_t axis;
    float pos;
    uint32_t L, m;
    uint32_t status;  // 1: the reference panics here
    uint32_t pad;
};

// Rust `f as usize` then min(7): saturating, NaN -> 0.
__device__ __forceinline__ uint32_t bin_of(float f) {
    if (!(f > 0.0f)) return 0u;
    if (f >= 7.0f) return 7u;
    return min(7u, (uint32_t)f);
}

__device__ __forceinline__ unsigned long long warp_min64(unsigned long long v) {
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long w = __shfl_xor_sync(0xFFFFFFFFu, v, o);
        v = w < v ? w : v;
    }
    return v;
}
__device__ __forceinline__ unsigned long long warp_max64(unsigned long long v) {
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long w = __shfl_xor_sync(0xFFFFFFFFu, v, o);
        v = w > v ? w : v;
    }
    return v;
}
__device__ __forceinline__ uint32_t warp_sum(uint32_t v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    return v;
}

// Block-wide min / max of N keys per thread, then one atomic per key into the node's slots.
template <int N>
__device__ __forceinline__ void flush_keys(const unsigned long long (&kmin)[N], const unsigned long long (&kmax)[N],
                                           unsigned long long* gmin, unsigned long long* gmax) {
    __shared__ unsigned long long smin[kThreads / 32][N], smax[kThreads / 32][N];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        const unsigned long long a = warp_min64(kmin[k]), b = warp_max64(kmax[k]);
        if (lane == 0) {
            smin[warp][k] = a;
            smax[warp][k] = b;
        }
    }
    __syncthreads();
    if (threadIdx.x < N) {
        unsigned long long a = kMinId, b = kMaxId;
        for (int w = 0; w < kThreads / 32; ++w) {
            a = smin[w][threadIdx.x] < a ? smin[w][threadIdx.x] : a;
            b = smax[w][threadIdx.x] > b ? smax[w][threadIdx.x] : b;
        }
        if (a != kMinId) atomicMin(&gmin[threadIdx.x], a);
        if (b != kMaxId) atomicMax(&gmax[threadIdx.x], b);
    }
}

// 1a. update_node_bounds: fold of every vertex component from (MAX, -MAX); order = 3 * pos + vertex.
__global__ void __launch_bounds__(kThreads) k_node_bounds(const Tile* __restrict__ tiles, const float* __restrict__ tris,
                                                          unsigned long long* kmin_g, unsigned long long* kmax_g) {
    const Tile t = tiles[blockIdx.x];
    unsigned long long kmin[3] = {kMinId, kMinId, kMinId}, kmax[3] = {kMaxId, kMaxId, kMaxId};
    for (uint32_t x = t.begin + threadIdx.x; x < t.end; x += kThreads) {
        const float* T = tris + 9ull * x;
#pragma unroll
        for (int v = 0; v < 3; ++v) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float f = T[3 * v + c];
                const uint32_t o = 3u * x + (uint32_t)v;
                if (f < FLT_MAX) kmin[c] = min(kmin[c], key_min(f, o));     // f32::min from MAX
                if (f > -FLT_MAX) kmax[c] = max(kmax[c], key_max(f, o));    // f32::max from -MAX
            }
        }
    }
    flush_keys<3>(kmin, kmax, kmin_g + (size_t)t.node * kKeysPerNode + kKeysNb,
                  kmax_g + (size_t)t.node * kKeysPerNode + kKeysNb);
}

// 1b. centroid bounds per axis: folds from 1e30 (min) and 1e-30 (max) (bvh.rs:339-340).
__global__ void __launch_bounds__(kThreads) k_cent_bounds(const Tile* __restrict__ tiles, const float* __restrict__ cent,
                                                          unsigned long long* kmin_g, unsigned long long* kmax_g) {
    const Tile t = tiles[blockIdx.x];
    unsigned long long kmin[3] = {kMinId, kMinId, kMinId}, kmax[3] = {kMaxId, kMaxId, kMaxId};
    for (uint32_t x = t.begin + threadIdx.x; x < t.end; x += kThreads) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float f = cent[3ull * x + c];
            if (f < 1e30f) kmin[c] = min(kmin[c], key_min(f, x));
            if (f > 1e-30f) kmax[c] = max(kmax[c], key_max(f, x));
        }
    }
    flush_keys<3>(kmin, kmax, kmin_g + (size_t)t.node * kKeysPerNode + kKeysCb,
                  kmax_g + (size_t)t.node * kKeysPerNode + kKeysCb);
}

__device__ __forceinline__ float vertex_comp(const float* tris, unsigned long long key, int c) {
    const uint32_t o = (uint32_t)(key & 0xFFFFFFFFull);
    return tris[9ull * (o / 3u) + 3u * (o % 3u) + (uint32_t)c];
}
__device__ __forceinline__ float vertex_comp_max(const float* tris, unsigned long long key, int c) {
    const uint32_t o = 0xFFFFFFFFu - (uint32_t)(key & 0xFFFFFFFFull);
    return tris[9ull * (o / 3u) + 3u * (o % 3u) + (uint32_t)c];
}

// 2. per node: decode node bounds and centroid bounds; binned axes and their scales.
__global__ void k_node_prep(LevelNode* nodes, uint32_t nact, const unsigned long long* kmin_g,
                            const unsigned long long* kmax_g, const float* __restrict__ tris,
                            const float* __restrict__ cent) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nact) return;
    LevelNode& nd = nodes[j];
    const unsigned long long* kn = kmin_g + (size_t)j * kKeysPerNode;
    const unsigned long long* kx = kmax_g + (size_t)j * kKeysPerNode;
    uint32_t active = 0;
    for (int c = 0; c < 3; ++c) {
        nd.lo[c] = kn[kKeysNb + c] != kMinId ? vertex_comp(tris, kn[kKeysNb + c], c) : FLT_MAX;
        nd.hi[c] = kx[kKeysNb + c] != kMaxId ? vertex_comp_max(tris, kx[kKeysNb + c], c) : -FLT_MAX;
        const unsigned long long a = kn[kKeysCb + c], b = kx[kKeysCb + c];
        const float cmin = a != kMinId ? cent[3ull * (uint32_t)(a & 0xFFFFFFFFull) + c] : 1e30f;
        const float cmax = b != kMaxId ? cent[3ull * (0xFFFFFFFFu - (uint32_t)(b & 0xFFFFFFFFull)) + c] : 1e-30f;
        nd.cmin[c] = cmin;
        nd.cmax[c] = cmax;
        nd.scale[c] = __fdiv_rn(8.0f, fsub(cmax, cmin));  // BINS / (bounds_max - bounds_min)
        if (!(cmin == cmax)) active |= 1u << c;
    }
    nd.active = active;
}

// 3. bins: count and the bin box grown from the zero box by each triangle's three vertices.
__global__ void __launch_bounds__(kThreads) k_bins(const Tile* __restrict__ tiles, const LevelNode* __restrict__ nodes,
                                                   const float* __restrict__ tris, const float* __restrict__ cent,
                                                   unsigned long long* kmin_g, unsigned long long* kmax_g,
                                                   uint32_t* cnt_g) {
    __shared__ uint32_t scnt[24];
    __shared__ unsigned long long smin[72], smax[72];
    const Tile t = tiles[blockIdx.x];
    const LevelNode& nd = nodes[t.node];
    for (int i = threadIdx.x; i < 72; i += kThreads) {
        smin[i] = kMinId;
        smax[i] = kMaxId;
        if (i < 24) scnt[i] = 0;
    }
    __syncthreads();
    const uint32_t active = nd.active;
    for (uint32_t x = t.begin + threadIdx.x; x < t.end; x += kThreads) {
        const float* T = tris + 9ull * x;
        for (int a = 0; a < 3; ++a) {
            if (!((active >> a) & 1u)) continue;
            const uint32_t b = bin_of(fmul(fsub(cent[3ull * x + a], nd.cmin[a]), nd.scale[a]));
            atomicAdd(&scnt[a * 8 + b], 1u);
#pragma unroll
            for (int v = 0; v < 3; ++v) {
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float f = T[3 * v + c];
                    const uint32_t o = 3u * x + (uint32_t)v;
                    const int slot = (a * 8 + (int)b) * 3 + c;
                    if (f < 0.0f) {  // f32::min from the zero box's +0
                        const unsigned long long k = key_min(f, o);
                        if (k < smin[slot]) atomicMin(&smin[slot], k);
                    }
                    if (f > 0.0f) {
                        const unsigned long long k = key_max(f, o);
                        if (k > smax[slot]) atomicMax(&smax[slot], k);
                    }
                }
            }
        }
    }
    __syncthreads();
    unsigned long long* gmin = kmin_g + (size_t)t.node * kKeysPerNode + kKeysBin;
    unsigned long long* gmax = kmax_g + (size_t)t.node * kKeysPerNode + kKeysBin;
    for (int i = threadIdx.x; i < 72; i += kThreads) {
        if (smin[i] != kMinId) atomicMin(&gmin[i], smin[i]);
        if (smax[i] != kMaxId) atomicMax(&gmax[i], smax[i]);
        if (i < 24 && scnt[i]) atomicAdd(&cnt_g[(size_t)t.node * 24 + i], scnt[i]);
    }
}

struct Box3 {
    float lo[3], hi[3];
};
__device__ __forceinline__ void box_zero(Box3& b) {
    for (int c = 0; c < 3; ++c) b.lo[c] = b.hi[c] = 0.0f;
}
__device__ __forceinline__ void box_grow(Box3& b, const float* p) {  // Aabb::grow (aabb.rs:36-39)
    for (int c = 0; c < 3; ++c) {
        b.lo[c] = min_ni(b.lo[c], p[c]);
        b.hi[c] = max_ni(b.hi[c], p[c]);
    }
}
__device__ __forceinline__ float box_area(const Box3& b) {  // Aabb::area (aabb.rs:48-57)
    const float ex = fsub(b.hi[0], b.lo[0]), ey = fsub(b.hi[1], b.lo[1]), ez = fsub(b.hi[2], b.lo[2]);
    return fadd(fadd(fmul(ex, ey), fmul(ey, ez)), fmul(ez, ex));
}

// 4. per node: the sweep, the split choice and the no-split test.
__global__ void k_node_split(LevelNode* nodes, uint32_t nact, const unsigned long long* kmin_g,
                             const unsigned long long* kmax_g, const uint32_t* cnt_g, const float* __restrict__ tris) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nact) return;
    LevelNode& nd = nodes[j];
    const unsigned long long* kn = kmin_g + (size_t)j * kKeysPerNode + kKeysBin;
    const unsigned long long* kx = kmax_g + (size_t)j * kKeysPerNode + kKeysBin;
    const uint32_t* cnt = cnt_g + (size_t)j * 24;
    int best_axis = -1;
    float best_pos = 0.0f, best_cost = FLT_MAX;
    for (int a = 0; a < 3; ++a) {
        if (!((nd.active >> a) & 1u)) continue;
        Box3 bins[8];
        for (int i = 0; i < 8; ++i) {
            for (int c = 0; c < 3; ++c) {
                const int s = (a * 8 + i) * 3 + c;
                bins[i].lo[c] = kn[s] != kMinId ? vertex_comp(tris, kn[s], c) : 0.0f;
                bins[i].hi[c] = kx[s] != kMaxId ? vertex_comp_max(tris, kx[s], c) : 0.0f;
            }
        }
        float la[7], ra[7];
        uint32_t lc[7], rc[7];
        Box3 lb, rb;
        box_zero(lb);
        box_zero(rb);
        uint32_t ls = 0, rs = 0;
        for (int i = 0; i < 7; ++i) {
            ls += cnt[a * 8 + i];
            lc[i] = ls;
            if (bins[i].lo[0] != FLT_MAX) {  // Aabb::grow_aabb (aabb.rs:41-46)
                box_grow(lb, bins[i].lo);
                box_grow(lb, bins[i].hi);
            }
            la[i] = box_area(lb);
            rs += cnt[a * 8 + 7 - i];
            rc[6 - i] = rs;
            if (bins[7 - i].lo[0] != FLT_MAX) {
                box_grow(rb, bins[7 - i].lo);
                box_grow(rb, bins[7 - i].hi);
            }
            ra[6 - i] = box_area(rb);
        }
        const float step = __fdiv_rn(fsub(nd.cmax[a], nd.cmin[a]), 8.0f);
        for (int i = 0; i < 7; ++i) {
            const float c = fadd(fmul(__uint2float_rn(lc[i]), la[i]), fmul(__uint2float_rn(rc[i]), ra[i]));
            if (c < best_cost) {
                best_axis = a;
                best_pos = fadd(nd.cmin[a], fmul(step, __int2float_rn(i + 1)));
                best_cost = c;
            }
        }
    }
    Box3 nb;
    for (int c = 0; c < 3; ++c) {
        nb.lo[c] = nd.lo[c];
        nb.hi[c] = nd.hi[c];
    }
    const float leaf_cost = fmul(__uint2float_rn(nd.count), box_area(nb));  // calculate_node_cost
    nd.axis = best_axis;
    nd.pos = best_pos;
    nd.attempt = !(best_cost >= leaf_cost) ? 1u : 0u;
    nd.status = (nd.attempt && best_axis < 0) ? 1u : 0u;
    nd.L = 0;
    nd.m = 0;
}

// 5a. the partition's test, cent[axis] < pos, and the number of left triangles per node.
__global__ void __launch_bounds__(kThreads) k_classify(const Tile* __restrict__ tiles, const LevelNode* nodes,
                                                       const float* __restrict__ cent, uint8_t* __restrict__ flag,
                                                       uint32_t* lcount) {
    __shared__ uint32_t sw[kThreads / 32];
    const Tile t = tiles[blockIdx.x];
    const LevelNode& nd = nodes[t.node];
    if (!nd.attempt) return;
    uint32_t n = 0;
    for (uint32_t x = t.begin + threadIdx.x; x < t.end; x += kThreads) {
        const bool left = cent[3ull * x + nd.axis] < nd.pos;
        flag[x] = left ? 1 : 0;
        n += left ? 1u : 0u;
    }
    n = warp_sum(n);
    if ((threadIdx.x & 31) == 0) sw[threadIdx.x >> 5] = n;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t s = 0;
        for (int w = 0; w < kThreads / 32; ++w) s += sw[w];
        if (s) atomicAdd(&lcount[t.node], s);
    }
}

// Per tile: right triangles in [first, first+L) and left ones in [first+L, end).
__global__ void __launch_bounds__(kThreads) k_tile_counts(const Tile* __restrict__ tiles, const LevelNode* nodes,
                                                          const uint32_t* lcount, const uint8_t* __restrict__ flag,
                                                          uint32_t* tile_fr, uint32_t* tile_bl) {
    __shared__ uint32_t sa[kThreads / 32], sb[kThreads / 32];
    const Tile t = tiles[blockIdx.x];
    const LevelNode& nd = nodes[t.node];
    if (!nd.attempt) return;
    const uint32_t split = nd.first + lcount[t.node];
    uint32_t fr = 0, bl = 0;
    for (uint32_t x = t.begin + threadIdx.x; x < t.end; x += kThreads) {
        const bool left = flag[x] != 0;
        fr += (x < split && !left) ? 1u : 0u;
        bl += (x >= split && left) ? 1u : 0u;
    }
    fr = warp_sum(fr);
    bl = warp_sum(bl);
    if ((threadIdx.x & 31) == 0) {
        sa[threadIdx.x >> 5] = fr;
        sb[threadIdx.x >> 5] = bl;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t a = 0, b = 0;
        for (int w = 0; w < kThreads / 32; ++w) {
            a += sa[w];
            b += sb[w];
        }
        tile_fr[blockIdx.x] = a;
        tile_bl[blockIdx.x] = b;
    }
}

// Per node: L, m, the tiles' rank offsets (right ones from the start, left ones from the end), and
// the reference's panic (an all-right partition of a node starting at 0 underflows its u32 index).
__global__ void k_node_offsets(LevelNode* nodes, uint32_t nact, const uint32_t* lcount, const uint32_t* tile_fr,
                               const uint32_t* tile_bl, uint32_t* tile_fr_off, uint32_t* tile_bl_off) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nact) return;
    LevelNode& nd = nodes[j];
    if (!nd.attempt) return;
    nd.L = lcount[j];
    uint32_t a = 0;
    for (uint32_t t = nd.tile_begin; t < nd.tile_end; ++t) {
        tile_fr_off[t] = a;
        a += tile_fr[t];
    }
    uint32_t b = 0;
    for (uint32_t t = nd.tile_end; t-- > nd.tile_begin;) {
        tile_bl_off[t] = b;
        b += tile_bl[t];
    }
    nd.m = a;
    if (a != b) nd.status = 2u;                // cannot happen: every left slot has one filler
    if (nd.first == 0 && nd.L == 0) nd.status = 1u;
}

// Block-wide exclusive scan of one value per thread.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* total) {
    __shared__ uint32_t sw[kThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t inc = v;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) sw[warp] = inc;
    __syncthreads();
    uint32_t base = 0, tot = 0;
    for (int w = 0; w < kThreads / 32; ++w) {
        if (w < warp) base += sw[w];
        tot += sw[w];
    }
    __syncthreads();
    *total = tot;
    return base + inc - v;
}

// Ranks: the k-th right triangle of [first, first+L) (k from 1) is recorded at rpos[first+k-1], the
// k-th left triangle of [first+L, end) counted from the end at lpos[first+k-1]; rank[x] keeps k.
// Each thread owns kPerThread consecutive triangles of the tile, so the block scans keep order.
__global__ void __launch_bounds__(kThreads) k_ranks(const Tile* __restrict__ tiles, const LevelNode* nodes,
                                                    const uint8_t* __restrict__ flag, const uint32_t* tile_fr_off,
                                                    const uint32_t* tile_bl_off, uint32_t* rank, uint32_t* rpos,
                                                    uint32_t* lpos) {
    const Tile t = tiles[blockIdx.x];
    const LevelNode& nd = nodes[t.node];
    if (!nd.attempt) return;
    const uint32_t split = nd.first + nd.L;
    const uint32_t x0 = t.begin + threadIdx.x * kPerThread;
    uint32_t fr = 0, bl = 0;
    for (uint32_t i = 0; i < kPerThread; ++i) {
        const uint32_t x = x0 + i;
        if (x >= t.end) break;
        const bool left = flag[x] != 0;
        fr += (x < split && !left) ? 1u : 0u;
        bl += (x >= split && left) ? 1u : 0u;
    }
    uint32_t fr_total, bl_total;
    uint32_t fr_before = block_excl_scan(fr, &fr_total);
    uint32_t bl_before = block_excl_scan(bl, &bl_total);
    const uint32_t fr_off = tile_fr_off[blockIdx.x], bl_off = tile_bl_off[blockIdx.x];
    uint32_t bl_incl = bl_before;
    for (uint32_t i = 0; i < kPerThread; ++i) {
        const uint32_t x = x0 + i;
        if (x >= t.end) break;
        const bool left = flag[x] != 0;
        if (x < split && !left) {
            const uint32_t k = fr_off + fr_before + 1u;
            fr_before += 1u;
            rank[x] = k;
            rpos[nd.first + k - 1u] = x;
        } else if (x >= split && left) {
            bl_incl += 1u;
            const uint32_t k = bl_off + (bl_total - bl_incl) + 1u;
            rank[x] = k;
            lpos[nd.first + k - 1u] = x;
        }
    }
}

// The scatter of the partition (closed form above); triangles, centroids and the permutation.
__global__ void __launch_bounds__(kThreads) k_scatter(const Tile* __restrict__ tiles, const LevelNode* nodes,
                                                      const uint8_t* __restrict__ flag, const uint32_t* rank,
                                                      const uint32_t* rpos, const uint32_t* lpos,
                                                      const float* __restrict__ tris_s, const float* __restrict__ cent_s,
                                                      const uint32_t* __restrict__ perm_s, float* __restrict__ tris_d,
                                                      float* __restrict__ cent_d, uint32_t* __restrict__ perm_d) {
    const Tile t = tiles[blockIdx.x];
    const LevelNode& nd = nodes[t.node];
    if (!nd.attempt || nd.status) return;
    const uint32_t first = nd.first, split = nd.first + nd.L, last = nd.first + nd.count - 1u, m = nd.m;
    for (uint32_t x = t.begin + threadIdx.x; x < t.end; x += kThreads) {
        const bool left = flag[x] != 0;
        uint32_t d;
        if (x < split) {
            if (left) {
                d = x;
            } else {
                const uint32_t k = rank[x];
                d = k == 1u ? last : lpos[first + k - 2u] - 1u;
            }
        } else if (left) {
            d = rpos[first + rank[x] - 1u];
        } else if (x == split) {
            d = m >= 1u ? lpos[first + m - 1u] - 1u : last;
        } else {
            d = x - 1u;
        }
        for (int c = 0; c < 9; ++c) tris_d[9ull * d + c] = tris_s[9ull * x + c];
        for (int c = 0; c < 3; ++c) cent_d[3ull * d + c] = cent_s[3ull * x + c];
        if (perm_s) perm_d[d] = perm_s[x];
    }
}

__global__ void __launch_bounds__(kThreads) k_copy_back(const Tile* __restrict__ tiles, const LevelNode* nodes,
                                                        const float* __restrict__ tris_d,
                                                        const float* __restrict__ cent_d,
                                                        const uint32_t* __restrict__ perm_d, float* __restrict__ tris_s,
                                                        float* __restrict__ cent_s, uint32_t* __restrict__ perm_s) {
    const Tile t = tiles[blockIdx.x];
    const LevelNode& nd = nodes[t.node];
    if (!nd.attempt || nd.status) return;
    for (uint32_t x = t.begin + threadIdx.x; x < t.end; x += kThreads) {
        for (int c = 0; c < 9; ++c) tris_s[9ull * x + c] = tris_d[9ull * x + c];
        for (int c = 0; c < 3; ++c) cent_s[3ull * x + c] = cent_d[3ull * x + c];
        if (perm_s) perm_s[x] = perm_d[x];
    }
}

// Triangle::centroid (triangle.rs:33-39): (v0 + v1 + v2) * (1/3), one/three in f32.
__global__ void k_centroids(const float* __restrict__ tris, uint32_t n, float* __restrict__ cent,
                            uint32_t* __restrict__ perm) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float third = __fdiv_rn(1.0f, fadd(fadd(1.0f, 1.0f), 1.0f));
    const float* T = tris + 9ull * i;
    for (int c = 0; c < 3; ++c) cent[3ull * i + c] = fmul(fadd(fadd(T[c], T[3 + c]), T[6 + c]), third);
    if (perm) perm[i] = i;
}

template <class T>
struct DevVec {
    T* p = nullptr;
    size_t cap = 0;
    cudaError_t reserve(size_t n) {
        if (n <= cap) return cudaSuccess;
        cudaFree(p);
        p = nullptr;
        cap = 0;
        cudaError_t e = cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T));
        if (e == cudaSuccess) cap = n;
        return e;
    }
    ~DevVec() { cudaFree(p); }
};

struct HostNode {  // one node of the level topology
    uint32_t first, count;
    float lo[3], hi[3];
    int64_t left = -1;  // index of the left child (the right one follows), -1 for a leaf
};

}  // namespace

int build_bvh_device(bvhgpu_ctx* ctx, float* mesh, uint32_t n, bvhgpu_node* nodes_out, uint32_t* nodes_used,
                     uint32_t* perm_out, const char** what) {
    *what = "";
    cudaStream_t s = ctx->stream;
    DevVec<float> tris[2], cent[2];
    DevVec<uint32_t> perm[2], rank, rpos, lpos;
    DevVec<uint8_t> flag;
#define BUILD_CK(expr, msg)                   \
    do {                                      \
        if ((expr) != cudaSuccess) {          \
            *what = msg;                      \
            return BVHGPU_ERR_CUDA;           \
        }                                     \
    } while (0)
    for (int b = 0; b < 2; ++b) {
        BUILD_CK(tris[b].reserve(9ull * n), "allocate triangles");
        BUILD_CK(cent[b].reserve(3ull * n), "allocate centroids");
        if (perm_out) BUILD_CK(perm[b].reserve(n), "allocate permutation");
    }
    BUILD_CK(rank.reserve(n), "allocate ranks");
    BUILD_CK(rpos.reserve(n), "allocate ranks");
    BUILD_CK(lpos.reserve(n), "allocate ranks");
    BUILD_CK(flag.reserve(n), "allocate flags");
    BUILD_CK(cudaMemcpyAsync(tris[0].p, mesh, 36ull * n, cudaMemcpyHostToDevice, s), "upload mesh");
    k_centroids<<<(n + 255) / 256, 256, 0, s>>>(tris[0].p, n, cent[0].p, perm_out ? perm[0].p : nullptr);
    g_launches++;
    BUILD_CK(cudaGetLastError(), "centroids");

    std::vector<HostNode> all;  // every node, level by level
    all.push_back(HostNode{0u, n, {0, 0, 0}, {0, 0, 0}, -1});
    size_t level_begin = 0, level_end = 1;
    DevVec<LevelNode> d_nodes;
    DevVec<Tile> d_tiles;
    DevVec<unsigned long long> d_kmin, d_kmax;
    DevVec<uint32_t> d_cnt, d_lcount, d_tfr, d_tbl, d_tfr_off, d_tbl_off;
    std::vector<LevelNode> lv;
    std::vector<Tile> tiles;
    while (level_begin < level_end) {
        const uint32_t nact = (uint32_t)(level_end - level_begin);
        lv.assign(nact, LevelNode{});
        tiles.clear();
        for (uint32_t j = 0; j < nact; ++j) {
            const HostNode& h = all[level_begin + j];
            lv[j].first = h.first;
            lv[j].count = h.count;
            lv[j].tile_begin = (uint32_t)tiles.size();
            for (uint32_t b = h.first; b < h.first + h.count; b += kTile)
                tiles.push_back(Tile{j, b, std::min(h.first + h.count, b + kTile), 0u});
            lv[j].tile_end = (uint32_t)tiles.size();
        }
        const uint32_t ntiles = (uint32_t)tiles.size();
        BUILD_CK(d_nodes.reserve(nact), "allocate level");
        BUILD_CK(d_tiles.reserve(ntiles), "allocate tiles");
        BUILD_CK(d_kmin.reserve((size_t)nact * kKeysPerNode), "allocate keys");
        BUILD_CK(d_kmax.reserve((size_t)nact * kKeysPerNode), "allocate keys");
        BUILD_CK(d_cnt.reserve((size_t)nact * 24), "allocate bins");
        BUILD_CK(d_lcount.reserve(nact), "allocate counts");
        BUILD_CK(d_tfr.reserve(ntiles), "allocate tile counts");
        BUILD_CK(d_tbl.reserve(ntiles), "allocate tile counts");
        BUILD_CK(d_tfr_off.reserve(ntiles), "allocate tile counts");
        BUILD_CK(d_tbl_off.reserve(ntiles), "allocate tile counts");
        BUILD_CK(cudaMemcpyAsync(d_nodes.p, lv.data(), sizeof(LevelNode) * nact, cudaMemcpyHostToDevice, s),
                 "upload level");
        BUILD_CK(cudaMemcpyAsync(d_tiles.p, tiles.data(), sizeof(Tile) * ntiles, cudaMemcpyHostToDevice, s),
                 "upload tiles");
        BUILD_CK(cudaMemsetAsync(d_kmin.p, 0xFF, sizeof(unsigned long long) * nact * kKeysPerNode, s), "keys");
        BUILD_CK(cudaMemsetAsync(d_kmax.p, 0x00, sizeof(unsigned long long) * nact * kKeysPerNode, s), "keys");
        BUILD_CK(cudaMemsetAsync(d_cnt.p, 0, sizeof(uint32_t) * nact * 24, s), "bins");
        BUILD_CK(cudaMemsetAsync(d_lcount.p, 0, sizeof(uint32_t) * nact, s), "counts");
        const unsigned nb = (nact + 127) / 128;
        k_node_bounds<<<ntiles, kThreads, 0, s>>>(d_tiles.p, tris[0].p, d_kmin.p, d_kmax.p);
        k_cent_bounds<<<ntiles, kThreads, 0, s>>>(d_tiles.p, cent[0].p, d_kmin.p, d_kmax.p);
        k_node_prep<<<nb, 128, 0, s>>>(d_nodes.p, nact, d_kmin.p, d_kmax.p, tris[0].p, cent[0].p);
        k_bins<<<ntiles, kThreads, 0, s>>>(d_tiles.p, d_nodes.p, tris[0].p, cent[0].p, d_kmin.p, d_kmax.p, d_cnt.p);
        k_node_split<<<nb, 128, 0, s>>>(d_nodes.p, nact, d_kmin.p, d_kmax.p, d_cnt.p, tris[0].p);
        k_classify<<<ntiles, kThreads, 0, s>>>(d_tiles.p, d_nodes.p, cent[0].p, flag.p, d_lcount.p);
        k_tile_counts<<<ntiles, kThreads, 0, s>>>(d_tiles.p, d_nodes.p, d_lcount.p, flag.p, d_tfr.p, d_tbl.p);
        k_node_offsets<<<nb, 128, 0, s>>>(d_nodes.p, nact, d_lcount.p, d_tfr.p, d_tbl.p, d_tfr_off.p, d_tbl_off.p);
        k_ranks<<<ntiles, kThreads, 0, s>>>(d_tiles.p, d_nodes.p, flag.p, d_tfr_off.p, d_tbl_off.p, rank.p, rpos.p,
                                            lpos.p);
        k_scatter<<<ntiles, kThreads, 0, s>>>(d_tiles.p, d_nodes.p, flag.p, rank.p, rpos.p, lpos.p, tris[0].p,
                                              cent[0].p, perm_out ? perm[0].p : nullptr, tris[1].p, cent[1].p,
                                              perm_out ? perm[1].p : nullptr);
        k_copy_back<<<ntiles, kThreads, 0, s>>>(d_tiles.p, d_nodes.p, tris[1].p, cent[1].p,
                                                perm_out ? perm[1].p : nullptr, tris[0].p, cent[0].p,
                                                perm_out ? perm[0].p : nullptr);
        g_launches += 12;
        BUILD_CK(cudaGetLastError(), "build level");
        BUILD_CK(cudaMemcpyAsync(lv.data(), d_nodes.p, sizeof(LevelNode) * nact, cudaMemcpyDeviceToHost, s),
                 "download level");
        BUILD_CK(cudaStreamSynchronize(s), "build level");
        const size_t next_begin = all.size();
        for (uint32_t j = 0; j < nact; ++j) {
            const LevelNode& d = lv[j];
            if (d.status) {
                *what = "the reference build panics on this mesh";
                return BVHGPU_ERR_BUILD;
            }
            HostNode& h = all[level_begin + j];
            std::memcpy(h.lo, d.lo, sizeof(h.lo));
            std::memcpy(h.hi, d.hi, sizeof(h.hi));
            if (d.attempt && d.L > 0 && d.L < d.count) {
                h.left = (int64_t)all.size();
                all.push_back(HostNode{d.first, d.L, {0, 0, 0}, {0, 0, 0}, -1});
                all.push_back(HostNode{d.first + d.L, d.count - d.L, {0, 0, 0}, {0, 0, 0}, -1});
            }
        }
        level_begin = next_begin;
        level_end = all.size();
    }
#undef BUILD_CK

    // the reference's depth-first numbering: splits counted per subtree, then pre-order ranks
    const size_t total = all.size();
    std::vector<uint32_t> splits(total, 0);
    for (size_t i = total; i-- > 0;)
        if (all[i].left >= 0) splits[i] = 1u + splits[all[i].left] + splits[all[i].left + 1];
    std::vector<uint32_t> pre(total, 0), index(total, 0);
    std::memset(nodes_out, 0, sizeof(bvhgpu_node) * 2ull * n);
    for (size_t i = 0; i < total; ++i) {  // parents come before children in `all`
        const HostNode& h = all[i];
        bvhgpu_node& o = nodes_out[index[i]];
        std::memcpy(o.bounds_min, h.lo, sizeof(h.lo));
        std::memcpy(o.bounds_max, h.hi, sizeof(h.hi));
        if (h.left < 0) {
            o.primitive_count = h.count;
            o.left_first = h.first;
            continue;
        }
        const size_t l = (size_t)h.left, r = l + 1;
        index[l] = 2u + 2u * pre[i];
        index[r] = 3u + 2u * pre[i];
        pre[l] = pre[i] + 1u;
        pre[r] = pre[i] + 1u + splits[l];
        o.primitive_count = 0;
        o.left_first = index[l];
    }
    *nodes_used = 2u + 2u * splits[0];
    if (cudaMemcpyAsync(mesh, tris[0].p, 36ull * n, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        (perm_out && cudaMemcpyAsync(perm_out, perm[0].p, 4ull * n, cudaMemcpyDeviceToHost, s) != cudaSuccess) ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        *what = "download the reordered mesh";
        return BVHGPU_ERR_CUDA;
    }
    return BVHGPU_OK;
}

}  // namespace bvhgpu
