// Ray traversal kernels: plain one-thread-per-ray BLAS traversal, the primary + diffuse
// bounce pipeline (plain and persistent), the uneven multi-scene batch (plain and
// persistent) and the tiled render.
//
// Persistent kernels: each warp keeps 32 ray slots; lanes whose ray finished are refilled
// together (ballot -> one atomicAdd per warp on a global queue -> shfl broadcast), so
// the SMs stay busy across scenes of very different sizes and across the incoherent
// bounce rays, and no lane idles while a neighbour finishes a long traversal.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <vector>

#include "common.cuh"
#include "internal.hpp"
#include "persistent.cuh"
#include "render.cuh"
#include "variants.cuh"

namespace bvhgpu {

namespace {

constexpr int kBlock = 128;
constexpr unsigned kFull = 0xFFFFFFFFu;
// Leaves with more triangles than this are tested by the whole warp (coop_leaf); smaller
// ones by the lane that reached them.

inline GBlas to_gblas(const DeviceBlas& b) {
    GBlas g;
    g.nodes = b.nodes;
    g.tris = b.tris;
    g.pairs = b.pairs;
    g.hx = b.hx;
    g.cones = b.cones;
    g.nodes_used = b.nodes_used;
    g.ntris = b.ntris;
    g.root_count = b.root_count;
    g.root_first = b.root_first;
    return g;
}

// Smallest compiled stack that holds `depth - 1` pending far children.
inline int stack_variant(uint32_t depth) {
    if (depth <= 33) return 32;
    if (depth <= 65) return 64;
    if (depth <= 129) return 128;
    return 256;
}

inline unsigned grid_for(uint32_t n, int block) { return (unsigned)((n + block - 1) / block); }

// ---- warp-synchronous traversal ----------------------------------------------------------
// Every lane walks its own ray through the interior nodes (and tests small leaves itself);
// a leaf with more than `pol.big_leaf` triangles (and no hidden tree walk) is tested by the whole warp together
// (coop_leaf), one waiting ray at a time.  All 32 lanes stay in the loop until every ray of
// the warp has finished, so the cooperative step always has the full warp.

// Traces the rays of one warp (inactive lanes take part in the cooperative steps only).
template <class STK>
__device__ __forceinline__ void warp_trace(const GBlas& b, bool active, LaneRay& r, LeafPolicy pol, uint32_t* err,
                                           uint2* stack_smem) {
    TravT<STK> tr;
    tr.stk.bind(stack_smem);
    if (active) tr.init(b);
    StepResult st = active ? kStepContinue : kStepFinished;
    for (;;) {
        if (st == kStepContinue) st = tr.template advance<true>(b, r, pol, err);
        unsigned pend = __ballot_sync(kFull, st == kStepBigLeaf);
        if (pend == 0u) break;
        coop_leaf_phase<true>(pend, b, tr, r, st);
    }
}

// ---- plain -------------------------------------------------------------------------------

// One thread per ray.  `count` (device, may be null) overrides n; `out_index` (may be null)
// maps ray i to its hit slot (the compacted bounce queue writes hits at pixel positions).
template <int BLOCK, int MINB, class STK>
__global__ void __launch_bounds__(BLOCK, MINB) k_trace_blas(GBlas b, const float4* __restrict__ rays, uint32_t n,
                                                            const uint32_t* count,
                                                            const uint32_t* __restrict__ out_index,
                                                            GHit* __restrict__ hits, LeafPolicy pol,
                                                            uint32_t* err) {
    extern __shared__ uint2 stack_smem[];
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (count) n = *count;
    if (__all_sync(kFull, i >= n)) return;  // whole warp idle
    bool active = i < n;
    LaneRay r;
    if (active) {
        float3 o, d;
        float t;
        load_ray(rays, i, o, d, t);
        init_lane_ray(r, o, d, t);
    }
    warp_trace<STK>(b, active, r, pol, err, stack_smem);
    // bvh.rs:295: a hit needs closest_ray.t < f32::MAX as well.
    if (active) store_hit(hits, out_index ? out_index[i] : i, r.hit && r.ct < FLT_MAX, r.ct, r.hu, r.hv, r.hp, 0u);
}

// The plain traversal with per-ray work counters (one variant: block 128, local stack), summed
// over the launch into out[0..6] in TraceCounts order -- the bytes each ray fetched, for the
// roofline.  Results are the same as k_trace_blas's.
__global__ void __launch_bounds__(kBlock) k_trace_count(GBlas b, const float4* __restrict__ rays, uint32_t n,
                                                        GHit* __restrict__ hits, LeafPolicy pol,
                                                        unsigned long long* out, uint32_t* err) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (__all_sync(kFull, i >= n)) return;
    const bool active = i < n;
    LaneRay r;
    if (active) {
        float3 o, d;
        float t;
        load_ray(rays, i, o, d, t);
        init_lane_ray(r, o, d, t);
    }
    TravT<LocalStack<256>, true> tr;
    tr.init(b);
    StepResult st = active ? kStepContinue : kStepFinished;
    for (;;) {
        if (st == kStepContinue) st = tr.template advance<true>(b, r, pol, err);
        const unsigned pend = __ballot_sync(kFull, st == kStepBigLeaf);
        if (pend == 0u) break;
        coop_leaf_phase(pend, b, tr, r, st);
    }
    if (active) store_hit(hits, i, r.hit && r.ct < FLT_MAX, r.ct, r.hu, r.hv, r.hp, 0u);
    if (!active) tr.cn = TraceCounts{0u, 0u, 0u, 0u, 0u, 0u, 0u};
    const uint32_t v[7] = {tr.cn.ref_nodes, tr.cn.hid_boxes, tr.cn.entries, tr.cn.hid_pairs, tr.cn.lane_tris,
                           tr.cn.coop_tris, tr.cn.cone_switches};
    for (int k = 0; k < 7; ++k) {
        unsigned long long s = v[k];
        for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(kFull, s, off);
        if ((threadIdx.x & 31u) == 0u && s) atomicAdd(out + k, s);
    }
}

// Bounce generation with warp-aggregated compaction: one atomicAdd per warp appends the
// warp's bounce rays to a dense queue (slot order is irrelevant: results go to pixels).
__global__ void __launch_bounds__(kBlock) k_bounce_gen(GBlas b, const float4* __restrict__ rays,
                                                       const GHit* __restrict__ hits0, uint32_t n, uint32_t seed,
                                                       float4* __restrict__ queue_rays, uint32_t* __restrict__ queue_pix,
                                                       uint32_t* queue_count, GHit* __restrict__ hits1, uint32_t key0) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    bool have = false;
    float3 po = make_float3(0, 0, 0), pd = make_float3(0, 0, 0);
    if (i < n) {
        GHit h = hits0[i];
        store_hit(hits1, i, false, 0, 0, 0, 0, 0);
        if (h.prim != kMiss) {
            float3 o, d;
            float t0;
            load_ray(rays, i, o, d, t0);
            const float4* T = b.tris + 3ull * h.prim;
            have = bounce_dir(o, d, h.t, __ldg(T), __ldg(T + 1), __ldg(T + 2), seed, key0 + i, po, pd);
        }
    }
    unsigned mask = __ballot_sync(kFull, have);
    if (mask == 0) return;
    unsigned lane = threadIdx.x & 31u;
    int leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if ((int)lane == leader) base = atomicAdd(queue_count, (uint32_t)__popc(mask));
    base = __shfl_sync(kFull, base, leader);
    if (have) {
        uint32_t slot = base + __popc(mask & ((1u << lane) - 1u));
        queue_rays[2ull * slot] = make_float4(po.x, po.y, po.z, FLT_MAX);
        queue_rays[2ull * slot + 1] = make_float4(pd.x, pd.y, pd.z, 0.0f);
        queue_pix[slot] = i;
    }
}

// Bounce rays in pixel order (for checking the bounce generation against the oracle).
__global__ void k_bounce_rays(GBlas b, const float4* __restrict__ rays, const GHit* __restrict__ hits0, uint32_t n,
                              uint32_t seed, float4* __restrict__ out, uint8_t* __restrict__ valid) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    GHit h = hits0[i];
    bool have = false;
    float3 po = make_float3(0, 0, 0), pd = make_float3(0, 0, 0);
    if (h.prim != kMiss) {
        float3 o, d;
        float t0;
        load_ray(rays, i, o, d, t0);
        const float4* T = b.tris + 3ull * h.prim;
        have = bounce_dir(o, d, h.t, __ldg(T), __ldg(T + 1), __ldg(T + 2), seed, i, po, pd);
    }
    out[2ull * i] = make_float4(po.x, po.y, po.z, FLT_MAX);
    out[2ull * i + 1] = make_float4(pd.x, pd.y, pd.z, 0.0f);
    valid[i] = have ? 1 : 0;
}

// Hit records with a primitive among hits[0, n), one atomicAdd per warp.
__global__ void k_count_hits(const GHit* __restrict__ hits, uint32_t n, uint32_t* count) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned m = __ballot_sync(kFull, i < n && hits[i].prim != kMiss);
    if ((threadIdx.x & 31u) == 0u && m) atomicAdd(count, (uint32_t)__popc(m));
}

// ---- persistent: primary + bounce in one launch -------------------------------------------
// Each warp keeps 32 ray slots.  A slot whose ray finished is refilled from the global queue
// (ballot -> one atomicAdd per warp -> shfl); a primary that hit continues in the same slot
// with its bounce ray, so no compaction pass and no second launch are needed.

template <int BLOCK, int MINB, class STK>
__global__ void __launch_bounds__(BLOCK, MINB) k_persistent_bounce(GBlas b, const float4* __restrict__ rays,
                                                                   uint32_t n, uint32_t seed,
                                                                   GHit* __restrict__ hits0, GHit* __restrict__ hits1,
                                                                   uint32_t* queue, LeafPolicy pol, uint32_t refill,
                                                                   uint32_t key0, uint32_t* hit_count, uint32_t* err) {
    extern __shared__ uint2 stack_smem[];
    const unsigned lane = threadIdx.x & 31u;
    int phase = 0;  // 0 needs work, 1 primary ray, 2 bounce ray, 3 retired
    uint32_t idx = 0;
    uint32_t nhit = 0;  // primary hits of this lane (summed into *hit_count at the end, if given)
    LaneRay r;
    TravT<STK> tr;
    tr.stk.bind(stack_smem);
    StepResult st = kStepFinished;
    bool queue_open = true;
    Deadline dl;
    dl.start(err);
    for (;;) {
        if (dl.expired(err)) return;
        const unsigned need = __ballot_sync(kFull, phase == 0);
        const unsigned busy = __ballot_sync(kFull, phase == 1 || phase == 2);
        // refill once `refill` lanes are idle (or none is busy)
        if (need != 0u && ((uint32_t)__popc(need) >= refill || busy == 0u)) {
            int leader = __ffs(need) - 1;
            uint32_t base = 0;
            if ((int)lane == leader) base = atomicAdd(queue, (uint32_t)__popc(need));
            base = __shfl_sync(kFull, base, leader);
            if (base + (uint32_t)__popc(need) >= n) queue_open = false;
            if (phase == 0) {
                uint32_t my = base + __popc(need & ((1u << lane) - 1u));
                if (my < n) {
                    idx = my;
                    float3 o, d;
                    float t0;
                    load_ray(rays, idx, o, d, t0);
                    init_lane_ray(r, o, d, t0);
                    tr.init(b);
                    st = kStepContinue;
                    phase = 1;
                } else {
                    phase = 3;
                }
            }
        }
        // advance this lane; finished rays are completed (a primary hit starts its bounce)
        while (phase == 1 || phase == 2) {
            if (st == kStepContinue) st = tr.advance(b, r, pol, err);
            if (st != kStepFinished) break;
            bool h = r.hit && r.ct < FLT_MAX;
            if (phase == 2) {
                store_hit(hits1, idx, h, r.ct, r.hu, r.hv, r.hp, 0u);
                phase = 0;
                break;
            }
            store_hit(hits0, idx, h, r.ct, r.hu, r.hv, r.hp, 0u);
            nhit += h ? 1u : 0u;
            float3 po, pd;
            bool have = false;
            if (h) {
                const float4* T = b.tris + 3ull * r.hp;
                have = bounce_dir(r.o, r.d, r.ct, __ldg(T), __ldg(T + 1), __ldg(T + 2), seed, key0 + idx, po, pd);
            }
            if (!have) {
                store_hit(hits1, idx, false, 0, 0, 0, 0, 0);
                phase = 0;
                break;
            }
            init_lane_ray(r, po, pd, FLT_MAX);
            tr.init(b);
            st = kStepContinue;
            phase = 2;
        }
        unsigned pend = __ballot_sync(kFull, (phase == 1 || phase == 2) && st == kStepBigLeaf);
        if (pend == 0u) {
            if (!queue_open && __ballot_sync(kFull, phase == 0 || phase == 1 || phase == 2) == 0u) {
                if (hit_count) {
                    for (int off = 16; off > 0; off >>= 1) nhit += __shfl_xor_sync(kFull, nhit, off);
                    if (lane == 0 && nhit) atomicAdd(hit_count, nhit);
                }
                break;
            }
            continue;
        }
        coop_leaf_phase(pend, b, tr, r, st);
    }
}

// ---- uneven batch ----------------------------------------------------------------------------

struct BatchEntry {
    GBlas blas;
    uint32_t ray_offset;
    uint32_t work_begin;  // prefix sum of ray counts
    uint32_t pad0, pad1;
};

template <int BLOCK, int MINB, class STK>
__global__ void __launch_bounds__(BLOCK, MINB) k_trace_batch_persistent(const BatchEntry* __restrict__ table,
                                                                        uint32_t nitems, uint32_t total,
                                                                        const float4* __restrict__ rays,
                                                                        GHit* __restrict__ hits, uint32_t* queue,
                                                                        LeafPolicy pol, uint32_t refill,
                                                                        uint32_t* err) {
    extern __shared__ uint2 stack_smem[];
    const unsigned lane = threadIdx.x & 31u;
    int phase = 0;  // 0 needs work, 1 tracing, 3 retired
    uint32_t ray = 0;
    GBlas b;
    b.nodes = nullptr;
    b.tris = nullptr;
    b.pairs = nullptr;
    b.hx = nullptr;
    b.cones = nullptr;
    b.nodes_used = b.ntris = b.root_count = b.root_first = 0;
    LaneRay r;
    TravT<STK> tr;
    tr.stk.bind(stack_smem);
    StepResult st = kStepFinished;
    bool queue_open = true;
    Deadline dl;
    dl.start(err);
    for (;;) {
        if (dl.expired(err)) return;
        const unsigned need = __ballot_sync(kFull, phase == 0);
        const unsigned busy = __ballot_sync(kFull, phase == 1);
        if (need != 0u && ((uint32_t)__popc(need) >= refill || busy == 0u)) {
            int leader = __ffs(need) - 1;
            uint32_t base = 0;
            if ((int)lane == leader) base = atomicAdd(queue, (uint32_t)__popc(need));
            base = __shfl_sync(kFull, base, leader);
            if (base + (uint32_t)__popc(need) >= total) queue_open = false;
            if (phase == 0) {
                uint32_t w = base + __popc(need & ((1u << lane) - 1u));
                if (w < total) {
                    uint32_t lo = 0, hi = nitems;  // last item with work_begin <= w
                    while (hi - lo > 1) {
                        uint32_t mid = (lo + hi) >> 1;
                        if (__ldg(&table[mid].work_begin) <= w) lo = mid; else hi = mid;
                    }
                    b = table[lo].blas;
                    ray = table[lo].ray_offset + (w - table[lo].work_begin);
                    float3 o, d;
                    float t0;
                    load_ray(rays, ray, o, d, t0);
                    init_lane_ray(r, o, d, t0);
                    tr.init(b);
                    st = kStepContinue;
                    phase = 1;
                } else {
                    phase = 3;
                }
            }
        }
        if (phase == 1) {
            if (st == kStepContinue) st = tr.advance(b, r, pol, err);
            if (st == kStepFinished) {
                store_hit(hits, ray, r.hit && r.ct < FLT_MAX, r.ct, r.hu, r.hv, r.hp, 0u);
                phase = 0;
            }
        }
        unsigned pend = __ballot_sync(kFull, phase == 1 && st == kStepBigLeaf);
        if (pend == 0u) {
            if (!queue_open && __ballot_sync(kFull, phase == 0 || phase == 1) == 0u) break;
            continue;
        }
        coop_leaf_phase<true>(pend, b, tr, r, st);
    }
}

// ---- triangle list, no BVH (Triangle::intersect / intersect_mut) ---------------------------
// One thread per ray; the block stages 128 triangles at a time in shared memory (each loaded
// once per block, then read by every lane) and tests them in index order.  Edges are formed on
// load with the single IEEE subtractions of triangle.rs:44-45 / 77-78.
//  kListClosest: Triangle::intersect with the strict `<` of a BVH leaf (first smallest t wins).
//  kListMut:     Triangle::intersect_mut on one Intersection per ray: each triangle that reports
//                a hit sets ray.t = min(ray.t, t) and overwrites u, v even when its t is larger.
constexpr int kListClosest = 0;
constexpr int kListMut = 1;
constexpr int kListTile = 128;

template <int MODE>
__global__ void __launch_bounds__(kListTile) k_triangle_list(const float* __restrict__ tris, uint32_t ntris,
                                                             const float4* __restrict__ rays, uint32_t n,
                                                             GHit* __restrict__ hits) {
    __shared__ float4 tile[3 * kListTile];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = i < n;
    float3 o = make_float3(0, 0, 0), d = o;
    float ct = FLT_MAX, hu = 0.0f, hv = 0.0f;
    uint32_t hp = kMiss;
    if (active) load_ray(rays, i, o, d, ct);
    for (uint32_t base = 0; base < ntris; base += kListTile) {
        __syncthreads();
        const uint32_t k = base + threadIdx.x;
        if (k < ntris) {
            const float* T = tris + 9ull * k;
            const float v0x = T[0], v0y = T[1], v0z = T[2];
            tile[3 * threadIdx.x] = make_float4(v0x, v0y, v0z, 0.0f);
            tile[3 * threadIdx.x + 1] = make_float4(fsub(T[3], v0x), fsub(T[4], v0y), fsub(T[5], v0z), 0.0f);
            tile[3 * threadIdx.x + 2] = make_float4(fsub(T[6], v0x), fsub(T[7], v0y), fsub(T[8], v0z), 0.0f);
        }
        __syncthreads();
        if (!active) continue;
        const uint32_t m = min((uint32_t)kListTile, ntris - base);
        for (uint32_t j = 0; j < m; ++j) {
            float t, u, v;
            if (!tri_test(tile[3 * j], tile[3 * j + 1], tile[3 * j + 2], o, d, t, u, v)) continue;
            if (MODE == kListClosest) {
                if (t < ct) {
                    ct = t;
                    hu = u;
                    hv = v;
                    hp = base + j;
                }
            } else {
                ct = min_ni(ct, t);
                hu = u;
                hv = v;
                hp = base + j;
            }
        }
    }
    if (active) store_hit(hits, i, hp != kMiss && (MODE == kListMut || ct < FLT_MAX), ct, hu, hv, hp, 0u);
}

// ---- tiled render --------------------------------------------------------------------------

// PathTracer::evaluate (renderer.rs:345-384): one 64-thread block per 8x8 tile; the camera ray
// goes through the pixel's top-left corner u = x / w, v = y / h (renderer.rs:358-361).  The
// normal accumulator's object transform is P.acc (16 floats).
template <int STACK>
__global__ void __launch_bounds__(64) k_render(GBlas b, RenderParams P, const float* __restrict__ normals,
                                               uint8_t* __restrict__ rgba, LeafPolicy pol, uint32_t* err) {
    const int tiles_x = (P.width + 7) / 8;
    const int tile = blockIdx.x;
    const int x = (tile % tiles_x) * 8 + (threadIdx.x & 7);
    const int y = (tile / tiles_x) * 8 + (threadIdx.x >> 3);
    const bool active = x < P.width && y < P.height;  // all lanes stay for the cooperative leaf steps
    float3 o, d;
    camera_ray(P, x, y, o, d);
    LaneRay lr;
    init_lane_ray(lr, o, d, FLT_MAX);
    warp_trace<LocalStack<STACK>>(b, active, lr, pol, err, nullptr);
    if (!active) return;
    const bool hit = lr.hit && lr.ct < FLT_MAX;
    const float3 rad = accumulate(P, hit, lr.ct, lr.hu, lr.hv, lr.hp, normals, P.acc, P.tex_coords, P.texels,
                                  P.tex_w, P.tex_h);
    reinterpret_cast<uchar4*>(rgba)[(size_t)y * P.width + x] = shade(P, rad);
}

}  // namespace

#define BVHGPU_DISPATCH_STACK(depth, ...)                         \
    switch (stack_variant(depth)) {                               \
        case 32: { constexpr int S = 32; __VA_ARGS__; break; }    \
        case 64: { constexpr int S = 64; __VA_ARGS__; break; }    \
        case 128: { constexpr int S = 128; __VA_ARGS__; break; }  \
        default: { constexpr int S = 256; __VA_ARGS__; break; }   \
    }

// Plain one-thread-per-ray launch; `count` (device) and `out_index` as in k_trace_blas.
static cudaError_t trace_blas_variant(bvhgpu_ctx* ctx, const Variant& v, const GBlas& g, const float4* rays,
                                      uint32_t n, const uint32_t* count, const uint32_t* out_index, GHit* hits,
                                      cudaStream_t s) {
    return with_variant(v.shape, v.stack, [&](auto sh, auto tg) {
        using SH = decltype(sh);
        using STK = typename decltype(tg)::type;
        k_trace_blas<SH::block, SH::minb, STK><<<grid_for(n, SH::block), SH::block,
                                                 stack_smem_bytes<STK>(SH::block), s>>>(g, rays, n, count, out_index,
                                                                                       hits, v.pol, ctx->d_err);
        return cudaGetLastError();
    });
}

cudaError_t launch_trace_blas(bvhgpu_ctx* ctx, const DeviceBlas& b, const float4* rays, uint32_t n, void* hits,
                              cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    GBlas g = to_gblas(b);
    LaunchScope scope(ctx, BVHGPU_K_TRACE_BLAS, s);
    const Variant v = resolve(ctx->tune[BVHGPU_K_TRACE_BLAS], b.depth);
    cudaError_t e = trace_blas_variant(ctx, v, g, rays, n, nullptr, nullptr, static_cast<GHit*>(hits), s);
    g_launches++;
    return e;
}

cudaError_t launch_bounce_plain(bvhgpu_ctx* ctx, const DeviceBlas& b, const float4* rays, uint32_t n, uint32_t seed,
                                void* hits0, void* hits1, cudaStream_t s, uint32_t base) {
    if (n == 0) return cudaSuccess;
    cudaError_t e = launch_trace_blas(ctx, b, rays, n, hits0, s);
    if (e != cudaSuccess) return e;
    uint32_t* qcount = ctx->d_scratch + 1;
    e = cudaMemsetAsync(qcount, 0, sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    GBlas g = to_gblas(b);
    {
        LaunchScope scope(ctx, BVHGPU_K_BOUNCE_GEN, s);
        k_bounce_gen<<<grid_for(n, kBlock), kBlock, 0, s>>>(g, rays, static_cast<const GHit*>(hits0), n, seed,
                                                            static_cast<float4*>(ctx->bounce_rays), ctx->bounce_pix,
                                                            qcount, static_cast<GHit*>(hits1), base);
        g_launches++;
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    {
        LaunchScope scope(ctx, BVHGPU_K_TRACE_QUEUE, s);
        const Variant v = resolve(ctx->tune[BVHGPU_K_TRACE_BLAS], b.depth);
        e = trace_blas_variant(ctx, v, g, static_cast<const float4*>(ctx->bounce_rays), n, qcount, ctx->bounce_pix,
                               static_cast<GHit*>(hits1), s);
        g_launches++;
    }
    return e;
}

cudaError_t launch_bounce_persistent(bvhgpu_ctx* ctx, const DeviceBlas& b, const float4* rays, uint32_t n,
                                     uint32_t seed, void* hits0, void* hits1, cudaStream_t s, uint32_t base,
                                     uint32_t* hit_count) {
    if (n == 0) return cudaSuccess;
    uint32_t* queue = ctx->d_scratch + 2;
    cudaError_t e = cudaMemsetAsync(queue, 0, sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    GBlas g = to_gblas(b);
    LaunchScope scope(ctx, BVHGPU_K_PERSISTENT_BOUNCE, s);
    const Variant v = resolve(ctx->tune[BVHGPU_K_PERSISTENT_BOUNCE], b.depth);
    e = with_variant(v.shape, v.stack, [&](auto sh, auto tg) {
        using SH = decltype(sh);
        using STK = typename decltype(tg)::type;
        auto* k = k_persistent_bounce<SH::block, SH::minb, STK>;
        const size_t smem = stack_smem_bytes<STK>(SH::block);
        k<<<persistent_grid(ctx, k, SH::block, smem), SH::block, smem, s>>>(
            g, rays, n, seed, static_cast<GHit*>(hits0), static_cast<GHit*>(hits1), queue, v.pol, v.refill, base,
            hit_count, ctx->d_err);
        return cudaGetLastError();
    });
    g_launches++;
    return e;
}

cudaError_t launch_trace_count(bvhgpu_ctx* ctx, const DeviceBlas& b, const float4* rays, uint32_t n, void* hits,
                               unsigned long long* out, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const Variant v = resolve(ctx->tune[BVHGPU_K_TRACE_BLAS], b.depth);
    LaunchScope scope(ctx, BVHGPU_K_OTHER, s);
    k_trace_count<<<grid_for(n, kBlock), kBlock, 0, s>>>(to_gblas(b), rays, n, static_cast<GHit*>(hits), v.pol, out,
                                                         ctx->d_err);
    g_launches++;
    return cudaGetLastError();
}

cudaError_t launch_count_hits(bvhgpu_ctx* ctx, const void* hits, uint32_t n, uint32_t* count, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    LaunchScope scope(ctx, BVHGPU_K_OTHER, s);
    k_count_hits<<<grid_for(n, 256), 256, 0, s>>>(static_cast<const GHit*>(hits), n, count);
    g_launches++;
    return cudaGetLastError();
}

cudaError_t launch_bounce_rays(bvhgpu_ctx* ctx, const DeviceBlas& b, const float4* rays, const void* hits0,
                               uint32_t n, uint32_t seed, float4* out, uint8_t* valid, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    GBlas g = to_gblas(b);
    LaunchScope scope(ctx, BVHGPU_K_OTHER, s);
    k_bounce_rays<<<grid_for(n, kBlock), kBlock, 0, s>>>(g, rays, static_cast<const GHit*>(hits0), n, seed, out,
                                                         valid);
    g_launches++;
    return cudaGetLastError();
}

bool batch_table_current(const bvhgpu_ctx* ctx, const bvhgpu_batch_item* items, uint32_t nitems) {
    return ctx->batch_items.size() == nitems && ctx->batch_table != nullptr &&
           std::equal(items, items + nitems, ctx->batch_items.begin(),
                      [](const bvhgpu_batch_item& a, const bvhgpu_batch_item& b) {
                          return a.blas == b.blas && a.ray_offset == b.ray_offset && a.ray_count == b.ray_count;
                      });
}

cudaError_t launch_trace_batch(bvhgpu_ctx* ctx, const std::vector<const DeviceBlas*>& blases,
                               const bvhgpu_batch_item* items, uint32_t nitems, const float4* rays, uint32_t nrays,
                               int mode, void* hits, cudaStream_t s) {
    (void)nrays;
    if (nitems == 0) return cudaSuccess;
    if (mode == BVHGPU_MODE_PLAIN) {
        for (uint32_t i = 0; i < nitems; ++i) {
            cudaError_t e = launch_trace_blas(ctx, *blases[i], rays + 2ull * items[i].ray_offset, items[i].ray_count,
                                              static_cast<GHit*>(hits) + items[i].ray_offset, s);
            if (e != cudaSuccess) return e;
        }
        return cudaSuccess;
    }
    // persistent: a device table of (BLAS, ray offset, work prefix), cached across calls
    if (!batch_table_current(ctx, items, nitems)) {
        std::vector<BatchEntry> table(nitems);
        uint32_t total = 0;
        uint32_t depth = 1;
        for (uint32_t i = 0; i < nitems; ++i) {
            table[i].blas = to_gblas(*blases[i]);
            table[i].ray_offset = items[i].ray_offset;
            table[i].work_begin = total;
            table[i].pad0 = table[i].pad1 = 0;
            total += items[i].ray_count;
            depth = std::max(depth, blases[i]->depth);
        }
        size_t bytes = sizeof(BatchEntry) * nitems;
        // the previous table may still be read by work queued on the stream
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return e;
        if (ctx->batch_table_bytes < bytes) {
            cudaFree(ctx->batch_table);
            ctx->batch_table = nullptr;
            ctx->batch_table_bytes = 0;
            e = cudaMalloc(&ctx->batch_table, bytes);
            if (e != cudaSuccess) return e;
            ctx->batch_table_bytes = bytes;
        }
        e = cudaMemcpy(ctx->batch_table, table.data(), bytes, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return e;
        ctx->batch_items.assign(items, items + nitems);
        ctx->batch_total = total;
        ctx->batch_depth = depth;
    }
    uint32_t* queue = ctx->d_scratch + 3;
    cudaError_t e = cudaMemsetAsync(queue, 0, sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    const uint32_t total = ctx->batch_total;
    LaunchScope scope(ctx, BVHGPU_K_TRACE_BATCH, s);
    const Variant v = resolve(ctx->tune[BVHGPU_K_TRACE_BATCH], ctx->batch_depth);
    e = with_variant(v.shape, v.stack, [&](auto sh, auto tg) {
        using SH = decltype(sh);
        using STK = typename decltype(tg)::type;
        auto* k = k_trace_batch_persistent<SH::block, SH::minb, STK>;
        const size_t smem = stack_smem_bytes<STK>(SH::block);
        k<<<persistent_grid(ctx, k, SH::block, smem), SH::block, smem, s>>>(
            static_cast<const BatchEntry*>(ctx->batch_table), nitems, total, rays, static_cast<GHit*>(hits), queue,
            v.pol, v.refill, ctx->d_err);
        return cudaGetLastError();
    });
    g_launches++;
    return e;
}

cudaError_t launch_triangle_list(bvhgpu_ctx* ctx, const float* tris, uint32_t ntris, const float4* rays, uint32_t n,
                                 int mode, void* hits, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    LaunchScope scope(ctx, BVHGPU_K_OTHER, s);
    if (mode == BVHGPU_LIST_MUT)
        k_triangle_list<kListMut><<<grid_for(n, kListTile), kListTile, 0, s>>>(tris, ntris, rays, n,
                                                                             static_cast<GHit*>(hits));
    else
        k_triangle_list<kListClosest><<<grid_for(n, kListTile), kListTile, 0, s>>>(tris, ntris, rays, n,
                                                                                 static_cast<GHit*>(hits));
    g_launches++;
    return cudaGetLastError();
}

cudaError_t launch_render(bvhgpu_ctx* ctx, const DeviceBlas& b, const bvhgpu_camera& cam, int w, int h, int acc,
                          const float* acc_params, int shader, const float* shader_params, const float* d_normals,
                          const float* d_tex_coords, const uint8_t* d_texels, uint32_t tex_w, uint32_t tex_h,
                          uint8_t* d_rgba, cudaStream_t s) {
    RenderParams P = make_render_params(cam, w, h, acc, acc_params, shader, shader_params);
    P.tex_coords = d_tex_coords;
    P.texels = d_texels;
    P.tex_w = tex_w;
    P.tex_h = tex_h;
    GBlas g = to_gblas(b);
    unsigned tiles = (unsigned)(((w + 7) / 8) * ((h + 7) / 8));
    LaunchScope scope(ctx, BVHGPU_K_RENDER, s);
    BVHGPU_DISPATCH_STACK(b.depth, (k_render<S><<<tiles, 64, 0, s>>>(g, P, d_normals, d_rgba, resolve(ctx->tune[BVHGPU_K_TRACE_BLAS], b.depth).pol, ctx->d_err)));
    g_launches++;
    return cudaGetLastError();
}

}  // namespace bvhgpu
