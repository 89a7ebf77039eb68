// BLAS vertex upload + refit, TLAS rebuild and instanced (two-level) traversal.
//
// Refit (Bvh::refit, bvh.rs:469-493): leaf boxes by a reduction over the triangles (exact
// order-preserving keys, so the min/max and its ties are the reference's), then the inner
// nodes bottom-up with one arrival counter per node: the second child to finish computes its
// parent with the reference's min/max order (left child first).
//
// TLAS rebuild (Tlas::rebuild, tlas.rs:204-250): the reference's agglomerative clustering with
// find_best_match results cached per list position in shared memory (see k_tlas_rebuild).
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "common.cuh"
#include "internal.hpp"
#include "render.cuh"
#include "variants.cuh"

namespace bvhgpu {
namespace {

constexpr int kBlock = 128;
constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr unsigned kFull = 0xFFFFFFFFu;

// Writes the traversal layout {v0, e1 = v1 - v0, e2 = v2 - v0} (the subtractions of
// triangle.rs:44-45, so no bit changes) and the raw vertices used by refit.
__global__ void k_write_tris(const float* __restrict__ tris9, uint32_t n, float4* __restrict__ out,
                             float4* __restrict__ verts, float* __restrict__ pairs) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* t = tris9 + 9ull * i;
    float4 v0 = make_float4(t[0], t[1], t[2], 0.0f);
    float4 v1 = make_float4(t[3], t[4], t[5], 0.0f);
    float4 v2 = make_float4(t[6], t[7], t[8], 0.0f);
    out[3ull * i] = v0;
    out[3ull * i + 1] = make_float4(fsub(v1.x, v0.x), fsub(v1.y, v0.y), fsub(v1.z, v0.z), 0.0f);
    out[3ull * i + 2] = make_float4(fsub(v2.x, v0.x), fsub(v2.y, v0.y), fsub(v2.z, v0.z), 0.0f);
    verts[3ull * i] = v0;
    verts[3ull * i + 1] = v1;
    verts[3ull * i + 2] = v2;
    // pair layout: component c of triangle i at float 20 * (i / 2) + 2c + (i & 1)
    float c[9] = {v0.x, v0.y, v0.z, fsub(v1.x, v0.x), fsub(v1.y, v0.y), fsub(v1.z, v0.z),
                  fsub(v2.x, v0.x), fsub(v2.y, v0.y), fsub(v2.z, v0.z)};
    float* P = pairs + 20ull * (i >> 1) + (i & 1u);
#pragma unroll
    for (int k = 0; k < 9; ++k) P[2 * k] = c[k];
}

// ---- hidden trees of the large leaves, refreshed after every triangle write -----------------
// Hidden pairs: the triangles of each pair's two slots (membership fixed at upload) copied into the
// packed layout.  Then one warp per hidden node and per cone record: the widened box of the
// node's pairs, or for a cone record the bounds Q, B and the normal cone of its pairs (cull.cuh).
__global__ void k_hidden_pairs(const float4* __restrict__ tris, const uint2* __restrict__ slots, uint32_t nhp,
                               float* __restrict__ pairs) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nhp) return;
    const uint2 idx = slots[j];
    float* P = pairs + 20ull * j;
    for (int h = 0; h < 2; ++h) {
        const uint32_t k = h ? idx.y : idx.x;
        float4 v0 = make_float4(0.0f, 0.0f, 0.0f, 0.0f), e1 = v0, e2 = v0;
        if (k != kMiss) {
            v0 = tris[3ull * k];
            e1 = tris[3ull * k + 1];
            e2 = tris[3ull * k + 2];
        }
        const float c[9] = {v0.x, v0.y, v0.z, e1.x, e1.y, e1.z, e2.x, e2.y, e2.z};
        for (int q = 0; q < 9; ++q) P[2 * q + h] = c[q];
    }
    P[18] = P[19] = 0.0f;
}

// The refresh runs over chunks of at most kRefreshChunk pairs, one warp each, so that the large
// groups near the hidden roots (up to ~10,000 pairs) are spread over many warps instead of
// holding one warp each for the whole launch.  A group's chunks are consecutive; the last chunk of
// a group to finish (arrival counter, reset by it) combines the group's partial results in chunk
// order, so every result is deterministic.  Pass 1 (k_hidden_refresh_boxes): the raw box
// aggregates of every group and, for cone groups, the sum of the sign-folded unit normals; a
// node group writes its widened box, a cone group its axis and the bounds Q, B.  Pass 2
// (k_hidden_refresh_cones, cone groups only): the cone's angle and the smallest normal, from the
// axis.  Min / max are exact in any order: boxes and cone angles do not depend on the chunking;
// the axis (a float sum) does, and any axis gives a valid cone.
__device__ __forceinline__ void agg_init(RefreshAgg& g) {
    for (int i = 0; i < 3; ++i) {
        g.lo[i] = FLT_MAX;
        g.hi[i] = -FLT_MAX;
    }
    g.e1m = g.e2m = 0.0f;
    g.sx = g.sy = g.sz = 0.0f;
    g.finite = true;
}

// Folds b into a: min / max of the bounds, sum of the normals.
__device__ __forceinline__ void agg_fold(RefreshAgg& a, const RefreshAgg& b) {
    for (int i = 0; i < 3; ++i) {
        a.lo[i] = fminf(a.lo[i], b.lo[i]);
        a.hi[i] = fmaxf(a.hi[i], b.hi[i]);
    }
    a.e1m = fmaxf(a.e1m, b.e1m);
    a.e2m = fmaxf(a.e2m, b.e2m);
    a.sx += b.sx;
    a.sy += b.sy;
    a.sz += b.sz;
    a.finite = a.finite && b.finite;
}

__device__ __forceinline__ RefreshAgg agg_shfl_xor(const RefreshAgg& g, int off) {
    RefreshAgg o;
    for (int i = 0; i < 3; ++i) {
        o.lo[i] = __shfl_xor_sync(0xFFFFFFFFu, g.lo[i], off);
        o.hi[i] = __shfl_xor_sync(0xFFFFFFFFu, g.hi[i], off);
    }
    o.e1m = __shfl_xor_sync(0xFFFFFFFFu, g.e1m, off);
    o.e2m = __shfl_xor_sync(0xFFFFFFFFu, g.e2m, off);
    o.sx = __shfl_xor_sync(0xFFFFFFFFu, g.sx, off);
    o.sy = __shfl_xor_sync(0xFFFFFFFFu, g.sy, off);
    o.sz = __shfl_xor_sync(0xFFFFFFFFu, g.sz, off);
    o.finite = __shfl_xor_sync(0xFFFFFFFFu, g.finite ? 1 : 0, off) != 0;
    return o;
}

// The warp's fold of every lane's aggregate (the same fixed tree on every lane).
__device__ __forceinline__ void agg_warp(RefreshAgg& g) {
    for (int off = 16; off > 0; off >>= 1) agg_fold(g, agg_shfl_xor(g, off));
}

// The first valid normal of a cone group in pair order (the sign reference of its folded normals).
__device__ __forceinline__ float3 group_reference_normal(const float* __restrict__ pairs, const uint2* __restrict__ slots,
                                                         uint32_t p0, uint32_t first, uint32_t end) {
    float rx = 0.0f, ry = 0.0f, rz = 0.0f;
    if ((threadIdx.x & 31u) == 0u) {
        for (uint32_t p = first; p < end; ++p) {
            const uint2 idx = slots[p - p0];
            const float* P = pairs + 20ull * p;
            bool found = false;
            for (int h = 0; h < 2 && !found; ++h) {
                if ((h ? idx.y : idx.x) == kMiss) continue;
                const float a[3] = {P[6 + h], P[8 + h], P[10 + h]}, b[3] = {P[12 + h], P[14 + h], P[16 + h]};
                rx = a[1] * b[2] - a[2] * b[1];
                ry = a[2] * b[0] - a[0] * b[2];
                rz = a[0] * b[1] - a[1] * b[0];
                found = isfinite(rx) && isfinite(ry) && isfinite(rz) && (rx != 0.0f || ry != 0.0f || rz != 0.0f);
            }
            if (found) break;
        }
    }
    return make_float3(__shfl_sync(0xFFFFFFFFu, rx, 0), __shfl_sync(0xFFFFFFFFu, ry, 0), __shfl_sync(0xFFFFFFFFu, rz, 0));
}

// Pass 1, one warp per chunk {group, first pair}.
__global__ void k_hidden_refresh_boxes(const uint4* __restrict__ work, const uint2* __restrict__ chunks, uint32_t nchunks,
                                       const uint32_t* __restrict__ chunk0, RefreshAgg* __restrict__ part,
                                       uint32_t* __restrict__ arrivals, const float* __restrict__ pairs,
                                       const uint2* __restrict__ slots, uint32_t p0, float4* __restrict__ nodes,
                                       float4* __restrict__ cones) {
    const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned lane = threadIdx.x & 31u;
    if (w >= nchunks) return;  // whole warps leave together
    const uint2 ch = chunks[w];
    const uint4 job = work[ch.x];
    const uint32_t end = min(ch.y + kRefreshChunk, job.y);
    const bool cone = job.w != kNoRefresh;
    RefreshAgg g;
    agg_init(g);
    for (uint32_t p = ch.y + lane; p < end; p += 32u) {
        const uint2 idx = slots[p - p0];
        const float* P = pairs + 20ull * p;
        for (int h = 0; h < 2; ++h) {
            if ((h ? idx.y : idx.x) == kMiss) continue;
            for (int i = 0; i < 3; ++i) {
                const float v = P[2 * i + h], a = P[2 * (3 + i) + h], b = P[2 * (6 + i) + h];
                const float p1 = fadd(v, a), p2 = fadd(v, b);
                g.finite = g.finite && isfinite(v) && isfinite(a) && isfinite(b) && isfinite(p1) && isfinite(p2);
                g.lo[i] = fminf(g.lo[i], fminf(v, fminf(p1, p2)));
                g.hi[i] = fmaxf(g.hi[i], fmaxf(v, fmaxf(p1, p2)));
                g.e1m = fmaxf(g.e1m, fabsf(a));
                g.e2m = fmaxf(g.e2m, fabsf(b));
            }
        }
    }
    if (cone) {
        // the sum of the unit normals, each turned towards the group's first one (any axis is
        // valid; this one makes the cone narrow)
        const float3 r = group_reference_normal(pairs, slots, p0, job.x, job.y);
        for (uint32_t p = ch.y + lane; p < end; p += 32u) {
            const uint2 idx = slots[p - p0];
            const float* P = pairs + 20ull * p;
            for (int h = 0; h < 2; ++h) {
                if ((h ? idx.y : idx.x) == kMiss) continue;
                const float a[3] = {P[6 + h], P[8 + h], P[10 + h]}, b[3] = {P[12 + h], P[14 + h], P[16 + h]};
                const float nx = a[1] * b[2] - a[2] * b[1], ny = a[2] * b[0] - a[0] * b[2], nz = a[0] * b[1] - a[1] * b[0];
                const float len = sqrtf(nx * nx + ny * ny + nz * nz);
                if (!(len > 0.0f) || !isfinite(len)) continue;
                const float sg = (nx * r.x + ny * r.y + nz * r.z) < 0.0f ? -1.0f : 1.0f;
                g.sx += sg * nx / len;
                g.sy += sg * ny / len;
                g.sz += sg * nz / len;
            }
        }
    }
    agg_warp(g);
    const uint32_t c0 = chunk0[ch.x], nc = chunk0[ch.x + 1] - c0;
    if (nc > 1) {
        // the group's last chunk to arrive combines the partials in chunk order
        bool last = false;
        if (lane == 0u) {
            part[w] = g;
            __threadfence();
            last = atomicAdd(arrivals + ch.x, 1u) == nc - 1u;
        }
        if (!__shfl_sync(0xFFFFFFFFu, last ? 1 : 0, 0)) return;
        __threadfence();
        agg_init(g);
        for (uint32_t k = lane; k < nc; k += 32u) {
            const RefreshAgg* q = part + c0 + k;
            RefreshAgg o;
            for (int i = 0; i < 3; ++i) {
                o.lo[i] = __ldcg(&q->lo[i]);
                o.hi[i] = __ldcg(&q->hi[i]);
            }
            o.e1m = __ldcg(&q->e1m);
            o.e2m = __ldcg(&q->e2m);
            o.sx = __ldcg(&q->sx);
            o.sy = __ldcg(&q->sy);
            o.sz = __ldcg(&q->sz);
            o.finite = *reinterpret_cast<volatile const bool*>(&q->finite);
            agg_fold(g, o);
        }
        agg_warp(g);
        if (lane == 0u) arrivals[ch.x] = 0u;  // ready for the next refresh
    }
    if (lane != 0u) return;
    const GroupSeal s = group_seal(g.lo, g.hi, g.e1m, g.e2m, g.finite);
    if (!cone) {  // a node's box
        float4* N = nodes + 2ull * job.z;
        N[0] = make_float4(s.lo[0], s.lo[1], s.lo[2], N[0].w);
        N[1] = make_float4(s.hi[0], s.hi[1], s.hi[2], N[1].w);
        return;
    }
    // the axis and the bounds Q, B, for pass 2
    float4* C = cones + 2ull * job.w;
    C[0] = make_float4(g.sx, g.sy, g.sz, 0.0f);
    C[1] = make_float4(0.0f, 0.0f, s.q, s.b);
}

// Pass 2, one warp per chunk of a cone group: the cone of the normal lines around the axis.
__global__ void k_hidden_refresh_cones(const uint4* __restrict__ work, const uint2* __restrict__ chunks,
                                       uint32_t first_chunk, uint32_t nchunks, const uint32_t* __restrict__ chunk0,
                                       float2* __restrict__ part, uint32_t* __restrict__ arrivals,
                                       const float* __restrict__ pairs, const uint2* __restrict__ slots, uint32_t p0,
                                       float4* __restrict__ cones) {
    const uint32_t w = first_chunk + ((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const unsigned lane = threadIdx.x & 31u;
    if (w >= nchunks) return;  // whole warps leave together
    const uint2 ch = chunks[w];
    const uint4 job = work[ch.x];
    const uint32_t end = min(ch.y + kRefreshChunk, job.y);
    float4* C = cones + 2ull * job.w;
    const float4 ax = __ldcg(C);
    float cmin = 2.0f, nmin = FLT_MAX;
    for (uint32_t p = ch.y + lane; p < end; p += 32u) {
        const uint2 idx = slots[p - p0];
        const float* P = pairs + 20ull * p;
        for (int h = 0; h < 2; ++h) {
            if ((h ? idx.y : idx.x) == kMiss) continue;
            const float a[3] = {P[6 + h], P[8 + h], P[10 + h]}, b[3] = {P[12 + h], P[14 + h], P[16 + h]};
            float cl, nl;
            cone_terms(a, b, ax.x, ax.y, ax.z, cl, nl);
            cmin = cl < cmin ? cl : (cl == cl ? cmin : -1.0f);  // NaN: no cone
            nmin = nl < nmin ? nl : (nl == nl ? nmin : 0.0f);
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        cmin = fminf(cmin, __shfl_xor_sync(0xFFFFFFFFu, cmin, off));
        nmin = fminf(nmin, __shfl_xor_sync(0xFFFFFFFFu, nmin, off));
    }
    const uint32_t c0 = chunk0[ch.x], nc = chunk0[ch.x + 1] - c0;
    if (nc > 1) {
        bool last = false;
        if (lane == 0u) {
            part[w] = make_float2(cmin, nmin);
            __threadfence();
            last = atomicAdd(arrivals + ch.x, 1u) == nc - 1u;
        }
        if (!__shfl_sync(0xFFFFFFFFu, last ? 1 : 0, 0)) return;
        __threadfence();
        cmin = 2.0f;
        nmin = FLT_MAX;
        for (uint32_t k = lane; k < nc; k += 32u) {
            const float2 q = __ldcg(part + c0 + k);
            cmin = fminf(cmin, q.x);
            nmin = fminf(nmin, q.y);
        }
        for (int off = 16; off > 0; off >>= 1) {
            cmin = fminf(cmin, __shfl_xor_sync(0xFFFFFFFFu, cmin, off));
            nmin = fminf(nmin, __shfl_xor_sync(0xFFFFFFFFu, nmin, off));
        }
        if (lane == 0u) arrivals[ch.x] = 0u;
    }
    if (lane != 0u) return;
    const float4 qb = __ldcg(C + 1);
    const bool cone_ok = isfinite(ax.x) && isfinite(ax.y) && isfinite(ax.z) && cmin > 0.0f && cmin <= 1.0f &&
                         nmin > 0.0f && nmin < FLT_MAX;
    C[0] = make_float4(cone_ok ? ax.x : 0.0f, cone_ok ? ax.y : 0.0f, cone_ok ? ax.z : 0.0f, cone_ok ? cmin : -1.0f);
    C[1] = make_float4(cone_ok ? cone_sin(cmin) : 1.0f, cone_ok ? nmin : 0.0f, qb.z, qb.w);
}

// ---- refit, parallel over triangles --------------------------------------------------------
// update_node_bounds (bvh.rs:317-330) folds a leaf's vertices in order v0, v1, v2 of triangle
// first, first+1, ... with f32::min / f32::max.  The fold's result is the minimum (maximum)
// value, and among equal values (only +0 / -0 differ in bits) the first one in that order.  The
// same result is computed in parallel with 64-bit keys: an order-preserving map of the value
// with both zeros mapped to one rank, then the position in the fold order (lower wins on a tie).
// NaNs are skipped, as f32::min skips them.  The reduced key names the winning vertex, whose
// actual bits are read back.

// Segmented min of 64-bit keys over consecutive lanes with the same segment id (leaf): the
// first lane of each segment ends up holding the segment's minimum.
__device__ __forceinline__ unsigned long long seg_min(unsigned long long k, uint32_t seg) {
    const unsigned lane = threadIdx.x & 31u;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        unsigned long long o = __shfl_down_sync(kFull, k, off);
        uint32_t os = __shfl_down_sync(kFull, seg, off);
        if (lane + off < 32u && os == seg && o < k) k = o;
    }
    return k;
}
__device__ __forceinline__ unsigned long long seg_max(unsigned long long k, uint32_t seg) {
    const unsigned lane = threadIdx.x & 31u;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        unsigned long long o = __shfl_down_sync(kFull, k, off);
        uint32_t os = __shfl_down_sync(kFull, seg, off);
        if (lane + off < 32u && os == seg && o > k) k = o;
    }
    return k;
}

constexpr unsigned long long kKeyMinIdentity = 0xFFFFFFFFFFFFFFFFull;
constexpr unsigned long long kKeyMaxIdentity = 0ull;

// One thread per triangle: keys of its three vertices per axis, reduced over the warp's lanes of
// the same leaf, then one atomicMin / atomicMax per (leaf, axis) from the segment's first lane.
// keys: 6 per leaf slot (min x y z, max x y z), at the identity before the launch.
__global__ void __launch_bounds__(256) k_refit_tris(const float4* __restrict__ verts, uint32_t ntris,
                                                    const uint32_t* __restrict__ tri_leaf,
                                                    unsigned long long* keys) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned lane = threadIdx.x & 31u;
    uint32_t slot = kNone;
    float4 v[3];
    if (i < ntris) {
        slot = tri_leaf[i];
        v[0] = verts[3ull * i];
        v[1] = verts[3ull * i + 1];
        v[2] = verts[3ull * i + 2];
    }
    const uint32_t prev = __shfl_up_sync(kFull, slot, 1);
    const bool head = slot != kNone && (lane == 0u || prev != slot);
#pragma unroll
    for (int axis = 0; axis < 3; ++axis) {
        unsigned long long kmin = kKeyMinIdentity, kmax = kKeyMaxIdentity;
        if (slot != kNone) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float x = axis == 0 ? v[c].x : (axis == 1 ? v[c].y : v[c].z);
                if (x != x) continue;
                const uint32_t pos = 3u * i + (uint32_t)c;
                const unsigned long long r = (unsigned long long)ordered(x) << 32;
                const unsigned long long a = r | pos, b = r | (0xFFFFFFFFu - pos);
                if (a < kmin) kmin = a;
                if (b > kmax) kmax = b;
            }
        }
        kmin = seg_min(kmin, slot);
        kmax = seg_max(kmax, slot);
        if (head) {
            if (kmin != kKeyMinIdentity) atomicMin(&keys[6ull * slot + axis], kmin);
            if (kmax != kKeyMaxIdentity) atomicMax(&keys[6ull * slot + 3 + axis], kmax);
        }
    }
}

// One thread per leaf: decode the keys into the winning vertices' values (identity = the fold's
// start value FLT_MAX / -FLT_MAX), reset the keys, write the leaf, then walk up: the second child
// to arrive at a parent computes it (bvh.rs:490-491: min(left, right), max(left, right)).
__global__ void __launch_bounds__(kBlock) k_refit_leaves(float4* nodes, const float4* __restrict__ verts,
                                                         const uint32_t* __restrict__ leaves, uint32_t nleaves,
                                                         const uint32_t* __restrict__ parent, uint32_t* counters,
                                                         unsigned long long* keys) {
    uint32_t li = blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= nleaves) return;
    const uint32_t ni = leaves[li];
    float b[6];
    for (int k = 0; k < 6; ++k) {
        const unsigned long long key = keys[6ull * li + k];
        const bool is_min = k < 3;
        keys[6ull * li + k] = is_min ? kKeyMinIdentity : kKeyMaxIdentity;
        if (key == (is_min ? kKeyMinIdentity : kKeyMaxIdentity)) {
            b[k] = is_min ? FLT_MAX : -FLT_MAX;
            continue;
        }
        uint32_t pos = (uint32_t)(key & 0xFFFFFFFFull);
        if (!is_min) pos = 0xFFFFFFFFu - pos;
        const float4 vv = verts[pos];  // pos = 3 * triangle + vertex indexes the float4 vertex array
        const int axis = k % 3;
        b[k] = axis == 0 ? vv.x : (axis == 1 ? vv.y : vv.z);
    }
    const float4 lo = nodes[2ull * ni], hi = nodes[2ull * ni + 1];
    nodes[2ull * ni] = make_float4(b[0], b[1], b[2], lo.w);
    nodes[2ull * ni + 1] = make_float4(b[3], b[4], b[5], hi.w);
    __threadfence();
    uint32_t p = parent[ni];
    while (p != kNone) {
        uint32_t old = atomicAdd(&counters[p], 1u);
        if (old == 0u) return;  // the sibling subtree is not done yet; it will continue
        counters[p] = 0u;
        __threadfence();
        float4 plo = __ldcg(&nodes[2ull * p]);
        float4 phi = __ldcg(&nodes[2ull * p + 1]);
        uint32_t l = __float_as_uint(plo.w);
        float4 llo = __ldcg(&nodes[2ull * l]), lhi = __ldcg(&nodes[2ull * l + 1]);
        float4 rlo = __ldcg(&nodes[2ull * l + 2]), rhi = __ldcg(&nodes[2ull * l + 3]);
        __stcg(&nodes[2ull * p], make_float4(min_ni(llo.x, rlo.x), min_ni(llo.y, rlo.y), min_ni(llo.z, rlo.z), plo.w));
        __stcg(&nodes[2ull * p + 1],
               make_float4(max_ni(lhi.x, rhi.x), max_ni(lhi.y, rhi.y), max_ni(lhi.z, rhi.z), phi.w));
        __threadfence();
        p = parent[p];
    }
}

// ---- TLAS ------------------------------------------------------------------------------------
// Tlas::rebuild (tlas.rs:204-250) walks nearest neighbours over a list of node indices and
// calls find_best_match (tlas.rs:179-202) -- a full scan of the list -- at every step.  Here
// each list position keeps the result find_best_match would give for it as one 64-bit key in
// shared memory: the area's order-preserving rank (both zeros one rank) above the position, so
// the smallest key is the smallest area with ties to the lower position, as the reference's
// strict `<` scan from FLT_MAX keeps it; areas not below FLT_MAX (and NaN) are never keys.  A
// merge updates only what it can change:
//  - the merged node lands on position a, the last node moves to position b, the list shrinks;
//  - a position whose cached best was a, b or the old last position is rescanned in full, by
//    several warps at once (each a slice of the list, combined with a shared-memory atomicMin);
//  - any other position keeps its cached best, which is still the first minimum over the
//    positions whose node did not change, and compares it with the two changed positions.
// The walk then reads the cache.  The TLAS is bit for bit Tlas::rebuild's, including the case
// where position a itself leaves the list (its stale entry is then scanned like a rescan).

constexpr int kTlasThreads = 512;
// Above this many objects the rebuild scans instead of caching each position's best match: the
// cache's rescans grow with the clusters (measured: 4,096 objects 2.5 s cached, 10 ms scanning;
// 256 objects, the instanced frame's, 0.46 ms cached, 0.61 ms scanning).
constexpr uint32_t kTlasCachedObjects = 256;
constexpr unsigned long long kNoKey = 0xFFFFFFFFFFFFFFFFull;

struct TlasSmem {  // one entry per list position
    unsigned long long* key;              // cached find_best_match(p)
    float *lx, *ly, *lz, *hx, *hy, *hz;  // node bounds (nodes[list[p]].aabb)
    int* node;                            // list[p]: node index
    int* inval;                           // positions to rescan after a merge
};

struct Box6 {
    float lx, ly, lz, hx, hy, hz;
};

__device__ __forceinline__ Box6 load_box(const TlasSmem& S, int p) {
    return Box6{S.lx[p], S.ly[p], S.lz[p], S.hx[p], S.hy[p], S.hz[p]};
}

// find_best_match's area (tlas.rs:184-193): component_max / component_min, then
// ex*ey + ey*ez + ez*ex.  The area is only compared (as a key rank), never stored, so fmaxf /
// fminf stand in for the first-operand-on-ties f32::max / f32::min: they ignore NaN the same way
// and can differ only in the sign of a zero coordinate, which changes at most the sign of a zero
// area -- the same rank.
__device__ __forceinline__ float sa_merge(const Box6& a, const TlasSmem& S, int r) {
    float ex = fsub(fmaxf(a.hx, S.hx[r]), fminf(a.lx, S.lx[r]));
    float ey = fsub(fmaxf(a.hy, S.hy[r]), fminf(a.ly, S.ly[r]));
    float ez = fsub(fmaxf(a.hz, S.hz[r]), fminf(a.lz, S.lz[r]));
    return fadd(fadd(fmul(ex, ey), fmul(ey, ez)), fmul(ez, ex));
}

// The cache key of candidate r for query box P (kNoKey where the reference would not take it).
__device__ __forceinline__ unsigned long long sa_key(const Box6& P, const TlasSmem& S, int r) {
    const float s = sa_merge(P, S, r);
    return s < FLT_MAX ? (((unsigned long long)ordered(s) << 32) | (uint32_t)r) : kNoKey;
}

__device__ __forceinline__ int key_pos(unsigned long long k) { return k == kNoKey ? -1 : (int)(uint32_t)k; }

// Warp minimum of 64-bit keys as two 32-bit warp reductions: the smallest high half (area rank),
// then the smallest low half (position) among the lanes holding that high half.
__device__ __forceinline__ unsigned long long warp_min_key(unsigned long long k) {
    const uint32_t hi = __reduce_min_sync(kFull, (uint32_t)(k >> 32));
    const uint32_t lo = __reduce_min_sync(kFull, (uint32_t)(k >> 32) == hi ? (uint32_t)k : 0xFFFFFFFFu);
    return ((unsigned long long)hi << 32) | lo;
}

// find_best_match for position p over positions [r0, r1) by one warp.
__device__ __forceinline__ unsigned long long warp_best_key(const TlasSmem& S, int p, int r0, int r1) {
    const Box6 P = load_box(S, p);
    unsigned long long best = kNoKey;
    for (int r = r0 + (int)(threadIdx.x & 31u); r < r1; r += 32) {
        if (r == p) continue;
        const unsigned long long k = sa_key(P, S, r);
        best = k < best ? k : best;
    }
    return warp_min_key(best);
}

__device__ __forceinline__ void xf_point_g(const float* m, float x, float y, float z, float* out) {
    out[0] = fadd(fadd(fadd(fmul(m[0], x), fmul(m[4], y)), fmul(m[8], z)), fmul(m[12], 1.0f));
    out[1] = fadd(fadd(fadd(fmul(m[1], x), fmul(m[5], y)), fmul(m[9], z)), fmul(m[13], 1.0f));
    out[2] = fadd(fadd(fadd(fmul(m[2], x), fmul(m[6], y)), fmul(m[10], z)), fmul(m[14], 1.0f));
}

__device__ __forceinline__ void store_tlas_node(float4* out, uint32_t i, const Box6& b, uint32_t left_right,
                                                uint32_t blas) {
    out[2ull * i] = make_float4(b.lx, b.ly, b.lz, __uint_as_float(left_right));
    out[2ull * i + 1] = make_float4(b.hx, b.hy, b.hz, __uint_as_float(blas));
}

// One merge of the walk by warp 0's lanes 0-6 (each touches only its own array): lane c < 6 the
// c-th coordinate array, lane 6 the node list.  Node `used` gets Aabb::new of positions a and b and
// LeftRightIndex::new(node a, node b) = a + (b << 16) (tlas.rs:18-22, 234-236); position a then
// holds it and position b the list's last node (tlas.rs:238-240).
__device__ __forceinline__ void tlas_merge(const TlasSmem& S, int n, float4* tlas_out, int a, int b, int last, int used,
                                           int lane) {
    if (lane >= 7) return;
    // node `used` as 8 floats: lo.xyz, left_right, hi.xyz, blas (0 for an inner node)
    float* out = reinterpret_cast<float*>(tlas_out) + 8ull * (uint32_t)used;
    if (lane < 6) {
        float* arr = S.lx + lane * n;  // lx, ly, lz, hx, hy, hz are consecutive arrays
        const float va = arr[a], vb = arr[b];
        const float m = lane < 3 ? min_ni(va, vb) : max_ni(va, vb);
        arr[a] = m;
        arr[b] = arr[last];
        out[lane < 3 ? lane : lane + 1] = m;
    } else {
        out[3] = __uint_as_float((uint32_t)S.node[a] + ((uint32_t)S.node[b] << 16));
        out[7] = __uint_as_float(0u);
        S.node[a] = used;
        S.node[b] = S.node[last];
    }
}

// One block.  Object world bounds (SceneObject::set_transform, scene_object.rs:60-75) in
// parallel, the cache filled one warp per position, then the walk: every thread follows it
// (it only reads the keys), warp 0 writes the merged nodes, all threads update the cache.
// status[0] gets nodes_used, status[1] an error (the reference would panic).  The per-position
// state lives in shared memory, or in `gwork` (global, same layout) for scenes too large for it.
__global__ void __launch_bounds__(kTlasThreads) k_tlas_rebuild(const GBlas* __restrict__ blas_table,
                                                               const uint32_t* __restrict__ obj_blas,
                                                               const float* __restrict__ xf, uint32_t nobj,
                                                               float4* __restrict__ tlas_out, uint32_t* status,
                                                               unsigned long long* gwork) {
    extern __shared__ unsigned long long tsm_keys[];
    __shared__ int s_ninval;
    __shared__ unsigned long long s_key_a;
    const int n = (int)nobj;
    TlasSmem S;
    S.key = gwork != nullptr ? gwork : tsm_keys;
    float* f = reinterpret_cast<float*>(S.key + n);
    S.lx = f;
    S.ly = f + n;
    S.lz = f + 2 * n;
    S.hx = f + 3 * n;
    S.hy = f + 4 * n;
    S.hz = f + 5 * n;
    S.node = reinterpret_cast<int*>(f + 6 * n);
    S.inval = reinterpret_cast<int*>(f + 7 * n);
    const int tid = (int)threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31, nwarps = (int)(blockDim.x >> 5);

    for (int i = tid; i < n; i += (int)blockDim.x) {
        const GBlas& b = blas_table[obj_blas[i]];
        float4 rlo = b.nodes[0], rhi = b.nodes[1];  // Bvh::bounds = nodes[0].aabb (bvh.rs:499-501)
        const float* m = xf + 16ull * i;
        float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
        float hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        for (int c = 0; c < 8; ++c) {
            float p[3];
            xf_point_g(m, (c & 1) ? rhi.x : rlo.x, (c & 2) ? rhi.y : rlo.y, (c & 4) ? rhi.z : rlo.z, p);
            for (int k = 0; k < 3; ++k) {
                lo[k] = min_ni(lo[k], p[k]);
                hi[k] = max_ni(hi[k], p[k]);
            }
        }
        S.lx[i] = lo[0];
        S.ly[i] = lo[1];
        S.lz[i] = lo[2];
        S.hx[i] = hi[0];
        S.hy[i] = hi[1];
        S.hz[i] = hi[2];
        S.node[i] = 1 + i;  // leaves at 1..nobj (tlas.rs:210-218)
        store_tlas_node(tlas_out, 1u + (uint32_t)i, Box6{lo[0], lo[1], lo[2], hi[0], hi[1], hi[2]}, 0u, (uint32_t)i);
    }
    __syncthreads();
    int count = n, used = 1 + n, a = 0;
    uint32_t err = 0;
    uint64_t steps = 0;
    const uint64_t max_steps = 4ull * nobj * nobj + 64;
    if (n > (int)kTlasCachedObjects) {
        // the reference's walk as written: every find_best_match a full scan by the block (no cache:
        // with many objects the merged clusters become the cached best of many positions, whose
        // rescans after each merge grow as n^2 per merge)
        auto best = [&](int p) {
            if (tid == 0) s_key_a = kNoKey;
            __syncthreads();
            const int chunk = (count + nwarps - 1) / nwarps;
            const int r0 = warp * chunk, r1 = min(count, r0 + chunk);
            if (r0 < r1) {
                const unsigned long long k = warp_best_key(S, p, r0, r1);
                if (lane == 0 && k != kNoKey) atomicMin(&s_key_a, k);
            }
            __syncthreads();
            const int r = key_pos(s_key_a);
            __syncthreads();
            return r;
        };
        int b = best(0);
        while (count > 1) {
            if (b < 0 || ++steps > max_steps) {
                err = 1;
                break;
            }
            const int c = best(b);
            if (a != c) {
                a = b;
                b = c;
                continue;
            }
            if (warp == 0) tlas_merge(S, n, tlas_out, a, b, count - 1, used, lane);
            count -= 1;
            used += 1;
            __syncthreads();
            b = best(a);
        }
        __syncthreads();
        if (tid == 0) {
            if (err == 0) {
                const uint32_t r = (uint32_t)S.node[a];
                const float4 r0 = tlas_out[2ull * r], r1 = tlas_out[2ull * r + 1];
                tlas_out[0] = r0;
                tlas_out[1] = r1;
            }
            status[0] = (uint32_t)used;
            status[1] = err;
        }
        return;
    }
    for (int p = warp; p < n; p += nwarps) {
        const unsigned long long k = warp_best_key(S, p, 0, n);
        if (lane == 0) S.key[p] = k;
    }
    __syncthreads();

    int b = key_pos(S.key[0]);
    while (count > 1) {
        if (b < 0 || ++steps > max_steps) {
            err = 1;
            break;
        }
        const int c = key_pos(S.key[b]);
        if (a != c) {
            a = b;
            b = c;
            continue;
        }
        const int last = count - 1;
        // Between the previous merge's last barrier and here the threads only read keys, so
        // warp 0 may rewrite the boxes and the node list right away.
        if (warp == 0) {
            tlas_merge(S, n, tlas_out, a, b, last, used, lane);
            if (lane == 6) s_ninval = 0;  // last read before the previous merge's final barrier
        }
        count = last;
        used += 1;
        __syncthreads();
        // s_key_a was read for the previous walk step by every thread before the barrier above
        if (tid == 0) s_key_a = kNoKey;
        for (int p = tid; p < count; p += (int)blockDim.x) {
            unsigned long long k = S.key[p];
            const int q = key_pos(k);
            if (p == a || p == b || q == a || q == b || q == last) {
                S.key[p] = kNoKey;
                S.inval[atomicAdd(&s_ninval, 1)] = p;
                continue;
            }
            const Box6 P = load_box(S, p);
            if (a < count) {
                const unsigned long long ka = sa_key(P, S, a);
                k = ka < k ? ka : k;
            }
            if (b < count) {
                const unsigned long long kb = sa_key(P, S, b);
                k = kb < k ? kb : k;
            }
            S.key[p] = k;
        }
        __syncthreads();
        // full rescans (and position a's stale entry if a left the list): every target split into
        // slices over the warps, slices combined with atomicMin
        const int ninval = s_ninval;
        const int ntarget = ninval + (a >= count ? 1 : 0);
        if (ntarget > 0) {
            const int slices = max(1, nwarps / ntarget);
            const int chunk = (count + slices - 1) / slices;
            for (int item = warp; item < ntarget * slices; item += nwarps) {
                const int j = item / slices, sl = item - j * slices;
                const int p = j < ninval ? S.inval[j] : a;
                const int r0 = sl * chunk, r1 = min(count, r0 + chunk);
                const unsigned long long k = warp_best_key(S, p, r0, r1);
                if (lane == 0 && k != kNoKey) atomicMin(j < ninval ? &S.key[p] : &s_key_a, k);
            }
        }
        __syncthreads();
        b = key_pos(a < count ? S.key[a] : s_key_a);
    }
    __syncthreads();  // the inner nodes written by warp 0's lanes are visible to thread 0
    if (tid == 0) {
        if (err == 0) {  // nodes[0] = nodes[list[a]] (tlas.rs:248)
            const uint32_t r = (uint32_t)S.node[a];
            const float4 r0 = tlas_out[2ull * r], r1 = tlas_out[2ull * r + 1];
            tlas_out[0] = r0;
            tlas_out[1] = r1;
        }
        status[0] = (uint32_t)used;
        status[1] = err;
    }
}

// ---- two-level traversal ------------------------------------------------------------------
// Tlas::intersect (tlas.rs:123-177) with SceneObject::intersect (scene_object.rs:78-89) at the
// leaves: the ray goes to model space through the cached inverse, 1/d' is recomputed (Ray::new)
// and the BLAS traversal (Trav, the same as for a single BLAS) shares the TLAS's closest t.  The
// LaneRay holds the model-space ray while a BLAS is traversed; the world ray is kept here.  Big
// BLAS leaves are handed to the warp-cooperative leaf phase, keyed by (BLAS, leaf), so rays in
// different instances of the same BLAS share the loaded triangle pairs.
struct SceneData {
    const float4* tlas;
    const GBlas* blas_table;
    const uint32_t* obj_blas;
    const float* inv;
    uint32_t tlas_nodes;
};

template <class STK, int TSTACK>
struct SceneTrav {
    TravT<STK> bt;
    GBlas blas;
    uint2 tstack[TSTACK];  // pending far TLAS nodes: (left_right, blas)
    int tsp;
    uint32_t lr, bl, tsteps;
    bool in_blas;
    float3 wo, wd, wrd;

    __device__ __forceinline__ void init(const SceneData& sd, LaneRay& r) {
        const float4 lo = __ldg(sd.tlas), hi = __ldg(sd.tlas + 1);
        lr = __float_as_uint(lo.w);
        bl = __float_as_uint(hi.w);
        tsp = 0;
        tsteps = 0;
        in_blas = false;
        wo = r.o;
        wd = r.d;
        wrd = r.rd;
        blas.nodes = nullptr;
        blas.tris = nullptr;
        blas.pairs = nullptr;
        blas.hx = nullptr;
        blas.cones = nullptr;
        blas.nodes_used = blas.ntris = blas.root_count = blas.root_first = 0;
    }

    __device__ __forceinline__ bool tpop() {
        if (tsp == 0) return true;
        --tsp;
        lr = tstack[tsp].x;
        bl = tstack[tsp].y;
        return false;
    }

    // After the cooperative test of the current big BLAS leaf.
    __device__ __forceinline__ StepResult after_leaf() {
        if (!bt.pop()) return kStepContinue;
        in_blas = false;
        return tpop() ? kStepFinished : kStepContinue;
    }

    __device__ __forceinline__ StepResult advance(const SceneData& sd, LaneRay& r, LeafPolicy pol, uint32_t* err) {
        for (;;) {
            if (in_blas) {
                const StepResult st = bt.step(blas, r, pol, err);
                if (st == kStepContinue) continue;
                if (st == kStepBigLeaf) return st;
                in_blas = false;
                if (tpop()) return kStepFinished;
                continue;
            }
            if (++tsteps > 2u * sd.tlas_nodes + 16u) {
                atomicOr(err, kErrSteps);
                return kStepFinished;
            }
            if (lr == 0u) {  // TLAS leaf: SceneObject::intersect
                const float* m = sd.inv + 16ull * bl;
                r.o.x = fadd(fadd(fadd(fmul(__ldg(m + 0), wo.x), fmul(__ldg(m + 4), wo.y)), fmul(__ldg(m + 8), wo.z)),
                             fmul(__ldg(m + 12), 1.0f));
                r.o.y = fadd(fadd(fadd(fmul(__ldg(m + 1), wo.x), fmul(__ldg(m + 5), wo.y)), fmul(__ldg(m + 9), wo.z)),
                             fmul(__ldg(m + 13), 1.0f));
                r.o.z = fadd(fadd(fadd(fmul(__ldg(m + 2), wo.x), fmul(__ldg(m + 6), wo.y)), fmul(__ldg(m + 10), wo.z)),
                             fmul(__ldg(m + 14), 1.0f));
                r.d.x = fadd(fadd(fadd(fmul(__ldg(m + 0), wd.x), fmul(__ldg(m + 4), wd.y)), fmul(__ldg(m + 8), wd.z)),
                             fmul(__ldg(m + 12), 0.0f));
                r.d.y = fadd(fadd(fadd(fmul(__ldg(m + 1), wd.x), fmul(__ldg(m + 5), wd.y)), fmul(__ldg(m + 9), wd.z)),
                             fmul(__ldg(m + 13), 0.0f));
                r.d.z = fadd(fadd(fadd(fmul(__ldg(m + 2), wd.x), fmul(__ldg(m + 6), wd.y)), fmul(__ldg(m + 10), wd.z)),
                             fmul(__ldg(m + 14), 0.0f));
                r.rd = recip3(r.d);
                r.inst_cur = bl;
                blas = sd.blas_table[__ldg(sd.obj_blas + bl)];
                bt.init(blas);
                in_blas = true;
                continue;
            }
            // LeftRightIndex getters are swapped (tlas.rs:24-32): left() is the high half.
            const uint32_t li = (lr & 0xFFFF0000u) >> 16, ri = lr & 0xFFFFu;
            const float4 l0 = __ldg(sd.tlas + 2ull * li), l1 = __ldg(sd.tlas + 2ull * li + 1);
            const float4 r0 = __ldg(sd.tlas + 2ull * ri), r1 = __ldg(sd.tlas + 2ull * ri + 1);
            float dl, dr;
            const bool hl = slab(l0, l1, wo, wrd, r.ct, dl);
            const bool hr = slab(r0, r1, wo, wrd, r.ct, dr);
            const float kl = hl ? dl : FLT_MAX;
            const float kr = hr ? dr : FLT_MAX;
            const bool left_near = kl < kr;
            const bool near_hit = left_near ? hl : hr;
            const bool far_hit = left_near ? hr : hl;
            if (near_hit) {
                if (far_hit) {
                    if (tsp >= TSTACK) {
                        atomicOr(err, kErrStack);
                        return kStepFinished;
                    }
                    tstack[tsp++] = left_near ? make_uint2(ubits(r0.w), ubits(r1.w)) : make_uint2(ubits(l0.w), ubits(l1.w));
                }
                lr = left_near ? ubits(l0.w) : ubits(r0.w);
                bl = left_near ? ubits(l1.w) : ubits(r1.w);
                continue;
            }
            if (tpop()) return kStepFinished;
        }
    }
};

// Cooperative phase of the two-level traversal (same grouping as the single-BLAS kernels).
template <class STK, int TSTACK>
__device__ __forceinline__ void scene_coop_phase(unsigned pend, SceneTrav<STK, TSTACK>& tr, LaneRay& r,
                                                 StepResult& st) {
    const unsigned lane = threadIdx.x & 31u;
    const unsigned long long key = reinterpret_cast<unsigned long long>(tr.blas.pairs);
    while (pend) {
        const int leader = __ffs(pend) - 1;
        const uint32_t f = __shfl_sync(kFull, tr.bt.first, leader);
        const uint32_t c = __shfl_sync(kFull, tr.bt.cnt, leader);
        const unsigned long long lk = __shfl_sync(kFull, key, leader);
        const ulonglong2* P = reinterpret_cast<const ulonglong2*>(lk);
        unsigned group = __ballot_sync(kFull, ((pend >> lane) & 1u) && tr.bt.first == f && key == lk);
        pend &= ~group;
        while (group) {
            const int a = __ffs(group) - 1;
            group &= group - 1u;
            if (group) {
                const int b = __ffs(group) - 1;
                group &= group - 1u;
                coop_leaf2(P, f, c, a, b, r);
                if ((int)lane == a || (int)lane == b) st = tr.after_leaf();
            } else {
                coop_leaf(P, f, c, a, r);
                if ((int)lane == a) st = tr.after_leaf();
            }
        }
    }
}

constexpr int kTlasStack = 64;

template <int BLOCK, int MINB, class STK>
__global__ void __launch_bounds__(BLOCK, MINB) k_trace_scene(SceneData sd, const float4* __restrict__ rays,
                                                             uint32_t n, GHit* __restrict__ hits, LeafPolicy pol,
                                                             uint32_t* err) {
    extern __shared__ uint2 stack_smem[];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (__all_sync(kFull, i >= n)) return;
    const bool active = i < n;
    LaneRay r;
    SceneTrav<STK, kTlasStack> tr;
    tr.bt.stk.bind(stack_smem);
    StepResult st = kStepFinished;
    if (active) {
        float3 o, d;
        float t0;
        load_ray(rays, i, o, d, t0);
        r.o = o;
        r.d = d;
        r.rd = recip3(d);
        r.ct = t0;
        r.hu = r.hv = 0.0f;
        r.hp = 0;
        r.hit = false;
        r.inst = r.inst_cur = 0;
        tr.init(sd, r);
        st = kStepContinue;
    }
    for (;;) {
        if (st == kStepContinue) st = tr.advance(sd, r, pol, err);
        const unsigned pend = __ballot_sync(kFull, st == kStepBigLeaf);
        if (pend == 0u) break;
        scene_coop_phase(pend, tr, r, st);
    }
    if (active) store_hit(hits, i, r.hit && r.ct < FLT_MAX, r.ct, r.hu, r.hv, r.hp, r.inst);
}

// PathTracer::evaluate over a whole scene (renderer.rs:345-384 -> Scene::intersect, scene.rs:32-34):
// one 64-thread block per 8x8 tile, the camera ray through the pixel's top-left corner, the two-level
// traversal of k_trace_scene, then the accumulator and shader.  The normal and texture accumulators
// look up `scene.get_unchecked(instance_index)` (renderer.rs:258-263, 312-317): with lookup 0 the
// reference's packed index -- instance 0, because Bvh::intersect packs instance 0
// (InstancePrimitiveIndex::from_primitive, bvh.rs:296), and the primitive's low 20 bits
// (intersection.rs:57-60) -- with lookup 1 the hit's own object.  A primitive outside the looked-up
// model's data (where the reference's slice indexing panics) or missing shading data sets kErrLookup
// and the pixel's radiance is zero.
template <int STACK>
__global__ void __launch_bounds__(64) k_render_scene(SceneData sd, RenderParams P,
                                                     const ShadeEntry* __restrict__ shade_tab,
                                                     const float* __restrict__ xf, int lookup,
                                                     uint8_t* __restrict__ rgba, LeafPolicy pol, uint32_t* err) {
    const int tiles_x = (P.width + 7) / 8;
    const int tile = blockIdx.x;
    const int x = (tile % tiles_x) * 8 + (threadIdx.x & 7);
    const int y = (tile / tiles_x) * 8 + (threadIdx.x >> 3);
    const bool active = x < P.width && y < P.height;  // all lanes stay for the cooperative leaf steps
    LaneRay r;
    SceneTrav<LocalStack<STACK>, kTlasStack> tr;
    tr.bt.stk.bind(nullptr);
    StepResult st = kStepFinished;
    if (active) {
        float3 o, d;
        camera_ray(P, x, y, o, d);
        r.o = o;
        r.d = d;
        r.rd = recip3(d);
        r.ct = FLT_MAX;
        r.hu = r.hv = 0.0f;
        r.hp = 0;
        r.hit = false;
        r.inst = r.inst_cur = 0;
        tr.init(sd, r);
        st = kStepContinue;
    }
    for (;;) {
        if (st == kStepContinue) st = tr.advance(sd, r, pol, err);
        const unsigned pend = __ballot_sync(kFull, st == kStepBigLeaf);
        if (pend == 0u) break;
        scene_coop_phase(pend, tr, r, st);
    }
    if (!active) return;
    const bool hit = r.hit && r.ct < FLT_MAX;
    const float* nrm = nullptr;
    const float* tc = nullptr;
    const uint8_t* tex = nullptr;
    uint32_t tw = 0, th = 0, prim = r.hp;
    const float* oxf = xf;
    bool ok = true;
    if (hit && (P.acc_kind == BVHGPU_ACC_NORMAL || P.acc_kind == BVHGPU_ACC_TEXTURE)) {
        const uint32_t obj = lookup ? r.inst : 0u;
        prim = lookup ? r.hp : (r.hp & 0x000FFFFFu);
        const ShadeEntry e = shade_tab[__ldg(sd.obj_blas + obj)];
        oxf = xf + 16ull * obj;
        nrm = e.normals;
        tc = e.tex_coords;
        tex = e.texels;
        tw = e.tex_w;
        th = e.tex_h;
        ok = prim < e.ntris && (P.acc_kind == BVHGPU_ACC_NORMAL ? nrm != nullptr
                                                                : (tc != nullptr && tex != nullptr && tw && th));
        if (!ok) atomicOr(err, kErrLookup);
    }
    const float3 rad = ok ? accumulate(P, hit, r.ct, r.hu, r.hv, prim, nrm, oxf, tc, tex, tw, th)
                          : make_float3(0.0f, 0.0f, 0.0f);
    reinterpret_cast<uchar4*>(rgba)[(size_t)y * P.width + x] = shade(P, rad);
}

// Persistent primary + bounce over a scene (the instanced frame): idle lanes are refilled from
// the queue; a primary that hits continues in its lane with the bounce ray of its hit.
template <int BLOCK, int MINB, class STK>
__global__ void __launch_bounds__(BLOCK, MINB) k_scene_persistent_bounce(SceneData sd, const float4* __restrict__ rays,
                                                                         uint32_t n, uint32_t seed,
                                                                         GHit* __restrict__ hits0,
                                                                         GHit* __restrict__ hits1, uint32_t* queue,
                                                                         LeafPolicy pol, uint32_t refill,
                                                                         uint32_t* err) {
    extern __shared__ uint2 stack_smem[];
    const unsigned lane = threadIdx.x & 31u;
    int phase = 0;  // 0 needs work, 1 primary, 2 bounce, 3 retired
    uint32_t idx = 0;
    LaneRay r;
    SceneTrav<STK, kTlasStack> tr;
    tr.bt.stk.bind(stack_smem);
    StepResult st = kStepFinished;
    bool queue_open = true;
    Deadline dl;
    dl.start(err);
    for (;;) {
        if (dl.expired(err)) return;
        const unsigned need = __ballot_sync(kFull, phase == 0);
        const unsigned busy = __ballot_sync(kFull, phase == 1 || phase == 2);
        if (need != 0u && ((uint32_t)__popc(need) >= refill || busy == 0u)) {
            const int leader = __ffs(need) - 1;
            uint32_t base = 0;
            if ((int)lane == leader) base = atomicAdd(queue, (uint32_t)__popc(need));
            base = __shfl_sync(kFull, base, leader);
            if (base + (uint32_t)__popc(need) >= n) queue_open = false;
            if (phase == 0) {
                const uint32_t my = base + __popc(need & ((1u << lane) - 1u));
                if (my < n) {
                    idx = my;
                    float3 o, d;
                    float t0;
                    load_ray(rays, idx, o, d, t0);
                    r.o = o;
                    r.d = d;
                    r.rd = recip3(d);
                    r.ct = t0;
                    r.hu = r.hv = 0.0f;
                    r.hp = 0;
                    r.hit = false;
                    r.inst = r.inst_cur = 0;
                    tr.init(sd, r);
                    st = kStepContinue;
                    phase = 1;
                } else {
                    phase = 3;
                }
            }
        }
        while (phase == 1 || phase == 2) {
            if (st == kStepContinue) st = tr.advance(sd, r, pol, err);
            if (st != kStepFinished) break;
            const bool h = r.hit && r.ct < FLT_MAX;
            if (phase == 2) {
                store_hit(hits1, idx, h, r.ct, r.hu, r.hv, r.hp, r.inst);
                phase = 0;
                break;
            }
            store_hit(hits0, idx, h, r.ct, r.hu, r.hv, r.hp, r.inst);
            float3 po, pd;
            bool have = false;
            if (h) {
                const GBlas hb = sd.blas_table[__ldg(sd.obj_blas + r.inst)];
                const float4* T = hb.tris + 3ull * r.hp;
                have = bounce_dir_instanced(tr.wo, tr.wd, r.ct, __ldg(T + 1), __ldg(T + 2), sd.inv + 16ull * r.inst,
                                            seed, idx, po, pd);
            }
            if (!have) {
                store_hit(hits1, idx, false, 0, 0, 0, 0, 0);
                phase = 0;
                break;
            }
            r.o = po;
            r.d = pd;
            r.rd = recip3(pd);
            r.ct = FLT_MAX;
            r.hu = r.hv = 0.0f;
            r.hp = 0;
            r.hit = false;
            r.inst = r.inst_cur = 0;
            tr.init(sd, r);
            st = kStepContinue;
            phase = 2;
        }
        const unsigned pend = __ballot_sync(kFull, (phase == 1 || phase == 2) && st == kStepBigLeaf);
        if (pend == 0u) {
            if (!queue_open && __ballot_sync(kFull, phase == 0 || phase == 1 || phase == 2) == 0u) break;
            continue;
        }
        scene_coop_phase(pend, tr, r, st);
    }
}

// Bounce rays of an instanced frame in pixel order (for checking against the oracle).
__global__ void k_scene_bounce_rays(SceneData sd, const float4* __restrict__ rays, const GHit* __restrict__ hits0,
                                    uint32_t n, uint32_t seed, float4* __restrict__ out, uint8_t* __restrict__ valid) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const GHit h = hits0[i];
    bool have = false;
    float3 po = make_float3(0, 0, 0), pd = po;
    if (h.prim != kMiss) {
        float3 o, d;
        float t0;
        load_ray(rays, i, o, d, t0);
        const GBlas hb = sd.blas_table[sd.obj_blas[h.inst]];
        const float4* T = hb.tris + 3ull * h.prim;
        have = bounce_dir_instanced(o, d, h.t, T[1], T[2], sd.inv + 16ull * h.inst, seed, i, po, pd);
    }
    out[2ull * i] = make_float4(po.x, po.y, po.z, FLT_MAX);
    out[2ull * i + 1] = make_float4(pd.x, pd.y, pd.z, 0.0f);
    valid[i] = have ? 1 : 0;
}

// ---- animation (the frame pattern of the reference's demos, closed form) --------------------
// Radial vertex wobble: v = dir * (r0 + amp * sin(freq * t + phase)), t read from device memory
// so that a captured frame graph replays with the current time.
__global__ void k_wobble(float* __restrict__ verts, const float* __restrict__ dirs, const float* __restrict__ r0,
                         const float* __restrict__ phase, uint32_t nv, float amp, float freq,
                         const float* __restrict__ time) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const float t = *time;
    const float r = r0[i] + amp * sinf(freq * t + phase[i]);
    verts[3ull * i] = dirs[3ull * i] * r;
    verts[3ull * i + 1] = dirs[3ull * i + 1] * r;
    verts[3ull * i + 2] = dirs[3ull * i + 2] * r;
}

// Instance i at time t: rotation R_i = R0_i * Rot(axis_i, omega_i t) (Rodrigues), uniform scale
// s_i, translation T_i; xf = [s R | T] and its inverse [R^T / s | -R^T T / s], column-major.
__global__ void k_animate_instances(float* __restrict__ xf, float* __restrict__ inv, const float* __restrict__ rot0,
                                    const float* __restrict__ axis, const float* __restrict__ omega,
                                    const float* __restrict__ scale, const float* __restrict__ trans, uint32_t n,
                                    const float* __restrict__ time) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float t = *time;
    const float ang = omega[i] * t;
    float sn, cs;
    sincosf(ang, &sn, &cs);
    const float kx = axis[3 * i], ky = axis[3 * i + 1], kz = axis[3 * i + 2];
    const float oc = 1.0f - cs;
    // Rot(axis, ang), row-major A[r][c]
    float A[3][3] = {{cs + kx * kx * oc, kx * ky * oc - kz * sn, kx * kz * oc + ky * sn},
                     {ky * kx * oc + kz * sn, cs + ky * ky * oc, ky * kz * oc - kx * sn},
                     {kz * kx * oc - ky * sn, kz * ky * oc + kx * sn, cs + kz * kz * oc}};
    const float* B = rot0 + 9ull * i;  // row-major R0
    float R[3][3];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) R[r][c] = B[3 * r] * A[0][c] + B[3 * r + 1] * A[1][c] + B[3 * r + 2] * A[2][c];
    const float s = scale[i], is = 1.0f / s;
    const float tx = trans[3 * i], ty = trans[3 * i + 1], tz = trans[3 * i + 2];
    float* X = xf + 16ull * i;
    float* I = inv + 16ull * i;
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) {
            X[4 * c + r] = s * R[r][c];
            I[4 * c + r] = is * R[c][r];
        }
    X[3] = X[7] = X[11] = 0.0f;
    X[12] = tx; X[13] = ty; X[14] = tz; X[15] = 1.0f;
    I[3] = I[7] = I[11] = 0.0f;
    for (int r = 0; r < 3; ++r) I[12 + r] = -(is * (R[0][r] * tx + R[1][r] * ty + R[2][r] * tz));
    I[15] = 1.0f;
}

__global__ void k_advance_time(float* time, float dt) { *time += dt; }

inline unsigned grid_for(uint32_t n, int block) { return (unsigned)((n + block - 1) / block); }

}  // namespace

cudaError_t launch_write_tris(bvhgpu_ctx* ctx, DeviceBlas& b, const float* d_tris9, cudaStream_t s) {
    if (b.ntris == 0) return cudaSuccess;
    LaunchScope scope(ctx, BVHGPU_K_OTHER, s);
    k_write_tris<<<grid_for(b.ntris, 256), 256, 0, s>>>(d_tris9, b.ntris, b.tris, b.verts,
                                                        reinterpret_cast<float*>(b.pairs));
    g_launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return launch_hidden_refresh(ctx, b, s);
}

cudaError_t launch_hidden_refresh(bvhgpu_ctx* ctx, DeviceBlas& b, cudaStream_t s) {
    if (b.nwork == 0) return cudaSuccess;
    LaunchScope scope(ctx, BVHGPU_K_OTHER, s);
    const uint32_t p0 = pairs_in_order(b.ntris);
    const uint2* slots = b.hx + hidden_table_u2(b.ntris);
    float* pairs = reinterpret_cast<float*>(b.pairs);
    k_hidden_pairs<<<grid_for(b.nhp, 256), 256, 0, s>>>(b.tris, slots, b.nhp, pairs + 20ull * p0);
    k_hidden_refresh_boxes<<<grid_for(32u * b.nchunks, 128), 128, 0, s>>>(
        b.hwork, b.hchunks, b.nchunks, b.hchunk0, static_cast<RefreshAgg*>(b.hpart), b.harrivals, pairs, slots, p0,
        b.nodes, b.cones);
    g_launches += 2;
    if (b.nchunks > b.nbox_chunks) {
        k_hidden_refresh_cones<<<grid_for(32u * (b.nchunks - b.nbox_chunks), 128), 128, 0, s>>>(
            b.hwork, b.hchunks, b.nbox_chunks, b.nchunks, b.hchunk0, static_cast<float2*>(b.hpart), b.harrivals,
            pairs, slots, p0, b.cones);
        g_launches++;
    }
    return cudaGetLastError();
}

cudaError_t launch_refit(bvhgpu_ctx* ctx, DeviceBlas& b, cudaStream_t s) {
    if (b.nleaves == 0) return cudaSuccess;
    LaunchScope scope(ctx, BVHGPU_K_REFIT, s);
    k_refit_tris<<<grid_for(b.ntris, 256), 256, 0, s>>>(b.verts, b.ntris, b.tri_leaf, b.leaf_keys);
    k_refit_leaves<<<grid_for(b.nleaves, kBlock), kBlock, 0, s>>>(b.nodes, b.verts, b.leaves, b.nleaves, b.parent,
                                                                  b.counters, b.leaf_keys);
    g_launches += 2;
    return cudaGetLastError();
}

size_t tlas_smem_bytes(uint32_t nobj) { return (8ull + 8ull * sizeof(float)) * nobj; }

cudaError_t launch_tlas_rebuild(bvhgpu_ctx* ctx, DeviceScene& sc, cudaStream_t s) {
    auto* gwork = static_cast<unsigned long long*>(sc.tlas_work);
    const size_t smem = gwork != nullptr ? 0 : tlas_smem_bytes(sc.nobjects);
    static bool attr_set = false;  // set outside graph capture: the first rebuild is scene_create's
    if (!attr_set) {
        cudaFuncSetAttribute(k_tlas_rebuild, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)tlas_smem_bytes(kTlasSharedObjects));
        attr_set = true;
    }
    LaunchScope scope(ctx, BVHGPU_K_TLAS_BUILD, s);
    k_tlas_rebuild<<<1, kTlasThreads, smem, s>>>(static_cast<const GBlas*>(sc.blas_table), sc.obj_blas, sc.xf,
                                                  sc.nobjects, sc.tlas, ctx->d_scratch + 8, gwork);
    g_launches++;
    return cudaGetLastError();
}

static SceneData scene_data(bvhgpu_ctx* ctx, DeviceScene& sc, uint32_t* depth) {
    SceneData sd;
    sd.tlas = sc.tlas;
    sd.blas_table = static_cast<const GBlas*>(sc.blas_table);
    sd.obj_blas = sc.obj_blas;
    sd.inv = sc.inv;
    sd.tlas_nodes = 2 * sc.nobjects;
    uint32_t d = 1;
    for (uint32_t id : sc.table_blas) d = std::max(d, ctx->blas[id].depth);
    *depth = d;
    return sd;
}

cudaError_t launch_trace_scene(bvhgpu_ctx* ctx, DeviceScene& sc, const float4* rays, uint32_t n, void* hits,
                               cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    uint32_t depth = 1;
    SceneData sd = scene_data(ctx, sc, &depth);
    LaunchScope scope(ctx, BVHGPU_K_TRACE_SCENE, s);
    const Variant v = resolve(ctx->tune[BVHGPU_K_TRACE_SCENE], depth);
    cudaError_t e = with_variant(v.shape, v.stack, [&](auto sh, auto tg) {
        using SH = decltype(sh);
        using STK = typename decltype(tg)::type;
        k_trace_scene<SH::block, SH::minb, STK><<<grid_for(n, SH::block), SH::block,
                                                  stack_smem_bytes<STK>(SH::block), s>>>(
            sd, rays, n, static_cast<GHit*>(hits), v.pol, ctx->d_err);
        return cudaGetLastError();
    });
    g_launches++;
    return e;
}

cudaError_t launch_render_scene(bvhgpu_ctx* ctx, DeviceScene& sc, const bvhgpu_camera& cam, int w, int h, int acc,
                                const float* acc_params, int shader, const float* shader_params,
                                const ShadeEntry* d_shade, int lookup, uint8_t* d_rgba, cudaStream_t s) {
    uint32_t depth = 1;
    SceneData sd = scene_data(ctx, sc, &depth);
    const RenderParams P = make_render_params(cam, w, h, acc, acc_params, shader, shader_params);
    const LeafPolicy pol = resolve(ctx->tune[BVHGPU_K_TRACE_SCENE], depth).pol;
    const unsigned tiles = (unsigned)(((w + 7) / 8) * ((h + 7) / 8));
    LaunchScope scope(ctx, BVHGPU_K_RENDER, s);
    // the smallest local stack that holds the deepest BLAS's pending far children
    if (depth <= 33)
        k_render_scene<32><<<tiles, 64, 0, s>>>(sd, P, d_shade, sc.xf, lookup, d_rgba, pol, ctx->d_err);
    else if (depth <= 65)
        k_render_scene<64><<<tiles, 64, 0, s>>>(sd, P, d_shade, sc.xf, lookup, d_rgba, pol, ctx->d_err);
    else if (depth <= 129)
        k_render_scene<128><<<tiles, 64, 0, s>>>(sd, P, d_shade, sc.xf, lookup, d_rgba, pol, ctx->d_err);
    else
        k_render_scene<256><<<tiles, 64, 0, s>>>(sd, P, d_shade, sc.xf, lookup, d_rgba, pol, ctx->d_err);
    g_launches++;
    return cudaGetLastError();
}

cudaError_t launch_scene_bounce(bvhgpu_ctx* ctx, DeviceScene& sc, const float4* rays, uint32_t n, uint32_t seed,
                                void* hits0, void* hits1, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    uint32_t depth = 1;
    SceneData sd = scene_data(ctx, sc, &depth);
    uint32_t* queue = ctx->d_scratch + 4;
    cudaError_t e = cudaMemsetAsync(queue, 0, sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    LaunchScope scope(ctx, BVHGPU_K_SCENE_BOUNCE, s);
    const Variant v = resolve(ctx->tune[BVHGPU_K_SCENE_BOUNCE], depth);
    e = with_variant(v.shape, v.stack, [&](auto sh, auto tg) {
        using SH = decltype(sh);
        using STK = typename decltype(tg)::type;
        auto* k = k_scene_persistent_bounce<SH::block, SH::minb, STK>;
        const size_t smem = stack_smem_bytes<STK>(SH::block);
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, SH::block, smem);
        k<<<std::max(1, per_sm) * ctx->num_sms, SH::block, smem, s>>>(sd, rays, n, seed, static_cast<GHit*>(hits0),
                                                                     static_cast<GHit*>(hits1), queue, v.pol,
                                                                     v.refill, ctx->d_err);
        return cudaGetLastError();
    });
    g_launches++;
    return e;
}

cudaError_t launch_scene_bounce_rays(bvhgpu_ctx* ctx, DeviceScene& sc, const float4* rays, const void* hits0,
                                     uint32_t n, uint32_t seed, float4* out, uint8_t* valid, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    uint32_t depth = 1;
    SceneData sd = scene_data(ctx, sc, &depth);
    LaunchScope scope(ctx, BVHGPU_K_OTHER, s);
    k_scene_bounce_rays<<<grid_for(n, kBlock), kBlock, 0, s>>>(sd, rays, static_cast<const GHit*>(hits0), n, seed,
                                                               out, valid);
    g_launches++;
    return cudaGetLastError();
}

cudaError_t launch_wobble(bvhgpu_ctx* ctx, float* verts, const float* dirs, const float* r0, const float* phase,
                          uint32_t nv, float amp, float freq, const float* time, cudaStream_t s) {
    LaunchScope scope(ctx, BVHGPU_K_OTHER, s);
    k_wobble<<<grid_for(nv, 256), 256, 0, s>>>(verts, dirs, r0, phase, nv, amp, freq, time);
    g_launches++;
    return cudaGetLastError();
}

cudaError_t launch_animate_instances(bvhgpu_ctx* ctx, DeviceScene& sc, const float* rot0, const float* axis,
                                     const float* omega, const float* scale, const float* trans, const float* time,
                                     cudaStream_t s) {
    LaunchScope scope(ctx, BVHGPU_K_OTHER, s);
    k_animate_instances<<<grid_for(sc.nobjects, 128), 128, 0, s>>>(sc.xf, sc.inv, rot0, axis, omega, scale, trans,
                                                                   sc.nobjects, time);
    g_launches++;
    return cudaGetLastError();
}

cudaError_t launch_advance_time(bvhgpu_ctx* ctx, float* time, float dt, cudaStream_t s) {
    LaunchScope scope(ctx, BVHGPU_K_OTHER, s);
    k_advance_time<<<1, 1, 0, s>>>(time, dt);
    g_launches++;
    return cudaGetLastError();
}

}  // namespace bvhgpu
