// BLAS vertex upload + refit, TLAS rebuild and instanced (two-level) traversal.
//
// Refit (Bvh::refit, bvh.rs:469-493) runs bottom-up with one thread per leaf and one
// arrival counter per node: the second child to finish computes its parent, so every
// node is written once, after both children, with the reference's min/max order
// (left child first).  The counters are reset by the thread that consumes them, so they
// are all zero again when the kernel ends.
//
// TLAS rebuild (Tlas::rebuild, tlas.rs:204-250) is the reference's agglomerative
// clustering itself, run by one warp over the nodes held in shared memory: each
// find_best_match (tlas.rs:179-202) is a warp-wide argmin, so the resulting TLAS is
// bit-identical to the reference's.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "common.cuh"
#include "internal.hpp"

namespace bvhgpu {
namespace {

constexpr int kBlock = 128;
constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr unsigned kFull = 0xFFFFFFFFu;

// f32::min / f32::max with the first operand kept on equality (same rule as the host build).
__device__ __forceinline__ float min_ni(float a, float b) {
    if (a != a) return b;
    if (b != b) return a;
    return (b < a) ? b : a;
}
__device__ __forceinline__ float max_ni(float a, float b) {
    if (a != a) return b;
    if (b != b) return a;
    return (b > a) ? b : a;
}

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

// ---- refit, parallel over triangles --------------------------------------------------------
// update_node_bounds (bvh.rs:317-330) folds a leaf's vertices in order v0, v1, v2 of triangle
// first, first+1, ... with f32::min / f32::max.  The fold's result is the minimum (maximum)
// value, and among equal values (only +0 / -0 differ in bits) the first one in that order.  The
// same result is computed in parallel with 64-bit keys: an order-preserving map of the value
// with both zeros mapped to one rank, then the position in the fold order (lower wins on a tie).
// NaNs are skipped, as f32::min skips them.  The reduced key names the winning vertex, whose
// actual bits are read back.
__device__ __forceinline__ uint32_t ordered(float f) {
    uint32_t b = __float_as_uint(f);
    if (f == 0.0f) return 0x80000000u;
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

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

struct SNode {  // shared-memory TLAS node
    float lo[3];
    float hi[3];
    uint32_t left_right;
    uint32_t blas;
};

__device__ __forceinline__ float sa_merge(const SNode& a, const SNode& b) {
    // find_best_match (tlas.rs:184-193): component_max / component_min with a's first
    float ex = fsub(max_ni(a.hi[0], b.hi[0]), min_ni(a.lo[0], b.lo[0]));
    float ey = fsub(max_ni(a.hi[1], b.hi[1]), min_ni(a.lo[1], b.lo[1]));
    float ez = fsub(max_ni(a.hi[2], b.hi[2]), min_ni(a.lo[2], b.lo[2]));
    return fadd(fadd(fmul(ex, ey), fmul(ey, ez)), fmul(ez, ex));
}

// Warp-wide find_best_match: the first b (in index order) with the strictly smallest
// surface area below FLT_MAX, or -1.
__device__ __forceinline__ int warp_best_match(const SNode* nodes, const int* list, int n, int a) {
    const unsigned lane = threadIdx.x & 31u;
    float best = FLT_MAX;
    int best_b = -1;
    const SNode& na = nodes[list[a]];
    for (int b = (int)lane; b < n; b += 32) {
        if (b == a) continue;
        float sa = sa_merge(na, nodes[list[b]]);
        if (sa < best) {
            best = sa;
            best_b = b;
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        float ob = __shfl_xor_sync(kFull, best, off);
        int obb = __shfl_xor_sync(kFull, best_b, off);
        bool take = (obb >= 0) && (best_b < 0 || ob < best || (ob == best && obb < best_b));
        if (take) {
            best = ob;
            best_b = obb;
        }
    }
    return best_b;
}

__device__ __forceinline__ void xf_point_g(const float* m, float x, float y, float z, float* out) {
    out[0] = fadd(fadd(fadd(fmul(m[0], x), fmul(m[4], y)), fmul(m[8], z)), fmul(m[12], 1.0f));
    out[1] = fadd(fadd(fadd(fmul(m[1], x), fmul(m[5], y)), fmul(m[9], z)), fmul(m[13], 1.0f));
    out[2] = fadd(fadd(fadd(fmul(m[2], x), fmul(m[6], y)), fmul(m[10], z)), fmul(m[14], 1.0f));
}

// One block: object world bounds (SceneObject::set_transform, scene_object.rs:60-75) in
// parallel, then warp 0 runs Tlas::rebuild.  status[0] gets nodes_used, status[1] an error.
__global__ void k_tlas_rebuild(const GBlas* __restrict__ blas_table, const uint32_t* __restrict__ obj_blas,
                               const float* __restrict__ xf, uint32_t nobj, float4* __restrict__ tlas_out,
                               uint32_t* status) {
    extern __shared__ unsigned char smem[];
    SNode* nodes = reinterpret_cast<SNode*>(smem);
    int* list = reinterpret_cast<int*>(nodes + 2 * nobj);
    for (uint32_t i = threadIdx.x; i < 2 * nobj; i += blockDim.x) {  // TlasNode::default
        SNode& s = nodes[i];
        s.lo[0] = s.lo[1] = s.lo[2] = FLT_MAX;
        s.hi[0] = s.hi[1] = s.hi[2] = -FLT_MAX;
        s.left_right = 0;
        s.blas = 0;
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < nobj; i += blockDim.x) {
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
        SNode& s = nodes[1 + i];  // leaves at 1..nobj (tlas.rs:210-218)
        for (int k = 0; k < 3; ++k) {
            s.lo[k] = lo[k];
            s.hi[k] = hi[k];
        }
        s.blas = i;
        s.left_right = 0;
        list[i] = (int)(1 + i);
    }
    __syncthreads();
    if (threadIdx.x >= 32) return;
    const unsigned lane = threadIdx.x;
    int count = (int)nobj;
    int used = 1 + (int)nobj;
    int a = 0;
    int b = warp_best_match(nodes, list, count, a);
    uint32_t err = 0;
    uint64_t iters = 0;
    const uint64_t max_iters = 4ull * nobj * nobj + 64;
    while (count > 1) {
        if (b < 0 || ++iters > max_iters) {
            err = 1;
            break;
        }
        int c = warp_best_match(nodes, list, count, b);
        if (a == c) {
            int ia = list[a], ib = list[b];
            if (lane == 0) {
                SNode na = nodes[ia], nb = nodes[ib];
                SNode& nn = nodes[used];
                nn.left_right = (uint32_t)ia + ((uint32_t)ib << 16);  // LeftRightIndex::new (tlas.rs:18-22)
                for (int k = 0; k < 3; ++k) {
                    nn.lo[k] = min_ni(na.lo[k], nb.lo[k]);
                    nn.hi[k] = max_ni(na.hi[k], nb.hi[k]);
                }
                list[a] = used;
                list[b] = list[count - 1];
            }
            __syncwarp();
            used += 1;
            count -= 1;
            b = warp_best_match(nodes, list, count, a);
        } else {
            if (c < 0) {
                err = 1;
                break;
            }
            a = b;
            b = c;
        }
    }
    __syncwarp();
    if (lane == 0 && err == 0) nodes[0] = nodes[list[a]];  // tlas.rs:248
    __syncwarp();
    for (uint32_t i = lane; i < 2 * nobj; i += 32) {
        const SNode& s = nodes[i];
        tlas_out[2ull * i] = make_float4(s.lo[0], s.lo[1], s.lo[2], __uint_as_float(s.left_right));
        tlas_out[2ull * i + 1] = make_float4(s.hi[0], s.hi[1], s.hi[2], __uint_as_float(s.blas));
    }
    if (lane == 0) {
        status[0] = (uint32_t)used;
        status[1] = err;
    }
}

// Tlas::intersect (tlas.rs:123-177) with SceneObject::intersect (scene_object.rs:78-89) at
// the leaves: the ray goes to model space through the cached inverse, 1/d' is recomputed
// (Ray::new), and the BLAS traversal shares the TLAS's closest t.
template <int STACK, int TSTACK>
__global__ void __launch_bounds__(kBlock) k_trace_scene(const float4* __restrict__ tlas,
                                                        const GBlas* __restrict__ blas_table,
                                                        const uint32_t* __restrict__ obj_blas,
                                                        const float* __restrict__ inv, const float4* __restrict__ rays,
                                                        uint32_t n, GHit* __restrict__ hits, uint32_t* err) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float3 o, d;
    float ct;
    load_ray(rays, i, o, d, ct);
    uint2 tstack[TSTACK];  // pending far TLAS nodes: (left_right, blas)
    int tsp = 0;
    float4 cur_lo = __ldg(tlas), cur_hi = __ldg(tlas + 1);
    uint32_t lr = __float_as_uint(cur_lo.w), bl = __float_as_uint(cur_hi.w);
    bool hit = false;
    float hu = 0.0f, hv = 0.0f;
    uint32_t hp = 0, hinst = 0;
    float3 rd = recip3(d);
    for (;;) {
        if (lr == 0u) {
            // leaf: SceneObject::intersect
            const float* m = inv + 16ull * bl;
            float3 mo, md;
            mo.x = fadd(fadd(fadd(fmul(__ldg(m + 0), o.x), fmul(__ldg(m + 4), o.y)), fmul(__ldg(m + 8), o.z)),
                        fmul(__ldg(m + 12), 1.0f));
            mo.y = fadd(fadd(fadd(fmul(__ldg(m + 1), o.x), fmul(__ldg(m + 5), o.y)), fmul(__ldg(m + 9), o.z)),
                        fmul(__ldg(m + 13), 1.0f));
            mo.z = fadd(fadd(fadd(fmul(__ldg(m + 2), o.x), fmul(__ldg(m + 6), o.y)), fmul(__ldg(m + 10), o.z)),
                        fmul(__ldg(m + 14), 1.0f));
            md.x = fadd(fadd(fadd(fmul(__ldg(m + 0), d.x), fmul(__ldg(m + 4), d.y)), fmul(__ldg(m + 8), d.z)),
                        fmul(__ldg(m + 12), 0.0f));
            md.y = fadd(fadd(fadd(fmul(__ldg(m + 1), d.x), fmul(__ldg(m + 5), d.y)), fmul(__ldg(m + 9), d.z)),
                        fmul(__ldg(m + 13), 0.0f));
            md.z = fadd(fadd(fadd(fmul(__ldg(m + 2), d.x), fmul(__ldg(m + 6), d.y)), fmul(__ldg(m + 10), d.z)),
                        fmul(__ldg(m + 14), 0.0f));
            GBlas b = blas_table[__ldg(obj_blas + bl)];
            float u2 = 0.0f, v2 = 0.0f;
            uint32_t p2 = 0;
            if (trace_blas<STACK>(b, mo, md, recip3(md), ct, u2, v2, p2, err)) {
                hit = true;
                hu = u2;
                hv = v2;
                hp = p2;
                hinst = bl;
            }
            if (tsp == 0) break;
            --tsp;
            lr = tstack[tsp].x;
            bl = tstack[tsp].y;
            continue;
        }
        // LeftRightIndex getters are swapped (tlas.rs:24-32): left() is the high half.
        uint32_t li = (lr & 0xFFFF0000u) >> 16, ri = lr & 0xFFFFu;
        float4 l0 = __ldg(tlas + 2ull * li), l1 = __ldg(tlas + 2ull * li + 1);
        float4 r0 = __ldg(tlas + 2ull * ri), r1 = __ldg(tlas + 2ull * ri + 1);
        float dl, dr;
        bool hl = slab(l0, l1, o, rd, ct, dl);
        bool hr = slab(r0, r1, o, rd, ct, dr);
        float kl = hl ? dl : FLT_MAX;
        float kr = hr ? dr : FLT_MAX;
        bool left_near = kl < kr;
        bool near_hit = left_near ? hl : hr;
        bool far_hit = left_near ? hr : hl;
        if (near_hit) {
            if (far_hit) {
                if (tsp >= TSTACK) {
                    atomicOr(err, kErrStack);
                    break;
                }
                tstack[tsp++] = left_near ? make_uint2(ubits(r0.w), ubits(r1.w)) : make_uint2(ubits(l0.w), ubits(l1.w));
            }
            lr = left_near ? ubits(l0.w) : ubits(r0.w);
            bl = left_near ? ubits(l1.w) : ubits(r1.w);
            continue;
        }
        if (tsp == 0) break;
        --tsp;
        lr = tstack[tsp].x;
        bl = tstack[tsp].y;
    }
    store_hit(hits, i, hit && ct < FLT_MAX, ct, hu, hv, hp, hinst);
}

inline unsigned grid_for(uint32_t n, int block) { return (unsigned)((n + block - 1) / block); }

}  // namespace

cudaError_t launch_write_tris(bvhgpu_ctx* ctx, DeviceBlas& b, const float* d_tris9, cudaStream_t s) {
    if (b.ntris == 0) return cudaSuccess;
    LaunchScope scope(ctx, BVHGPU_K_OTHER, s);
    k_write_tris<<<grid_for(b.ntris, 256), 256, 0, s>>>(d_tris9, b.ntris, b.tris, b.verts,
                                                        reinterpret_cast<float*>(b.pairs));
    g_launches++;
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

size_t tlas_smem_bytes(uint32_t nobj) { return sizeof(SNode) * 2ull * nobj + sizeof(int) * nobj; }

cudaError_t launch_tlas_rebuild(bvhgpu_ctx* ctx, DeviceScene& sc, cudaStream_t s) {
    size_t smem = tlas_smem_bytes(sc.nobjects);
    static bool attr_set = false;
    if (!attr_set) {
        cudaFuncSetAttribute(k_tlas_rebuild, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        attr_set = true;
    }
    LaunchScope scope(ctx, BVHGPU_K_TLAS_BUILD, s);
    k_tlas_rebuild<<<1, 256, smem, s>>>(static_cast<const GBlas*>(sc.blas_table), sc.obj_blas, sc.xf, sc.nobjects,
                                        sc.tlas, ctx->d_scratch + 8);
    g_launches++;
    return cudaGetLastError();
}

cudaError_t launch_trace_scene(bvhgpu_ctx* ctx, DeviceScene& sc, const float4* rays, uint32_t n, void* hits,
                               cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    uint32_t depth = 1;
    for (uint32_t id : sc.table_blas) depth = std::max(depth, ctx->blas[id].depth);
    LaunchScope scope(ctx, BVHGPU_K_TRACE_SCENE, s);
    const GBlas* table = static_cast<const GBlas*>(sc.blas_table);
    GHit* h = static_cast<GHit*>(hits);
    unsigned grid = grid_for(n, kBlock);
    if (depth <= 33)
        k_trace_scene<32, 64><<<grid, kBlock, 0, s>>>(sc.tlas, table, sc.obj_blas, sc.inv, rays, n, h, ctx->d_err);
    else if (depth <= 65)
        k_trace_scene<64, 64><<<grid, kBlock, 0, s>>>(sc.tlas, table, sc.obj_blas, sc.inv, rays, n, h, ctx->d_err);
    else
        k_trace_scene<256, 64><<<grid, kBlock, 0, s>>>(sc.tlas, table, sc.obj_blas, sc.inv, rays, n, h, ctx->d_err);
    g_launches++;
    return cudaGetLastError();
}

}  // namespace bvhgpu
