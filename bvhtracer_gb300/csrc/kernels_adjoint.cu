// Differentiable Lambertian render on an indexed mesh (not in the reference).
//
// Forward, per camera ray: closest hit through the reference-built BLAS (same traversal as
// every other trace), hit record {t, u, v, prim} checkpointed, and
//     p = o + d t,  l = L - p,  n = n0 (1 - u - v) + n1 u + n2 v  (renderer.rs:268-272),
//     I = max(0, normalize(n) . normalize(l))
// with the vertex normals n_i held fixed.  Adjoint, per pixel, from the checkpointed record
// (no re-trace, visibility fixed): dLoss/dI -> dI/d(t, u, v) -> vertices.  For the
// Moeller-Trumbore solution x = (t, u, v) of M x = o - v0 with M = [-d | e1 | e2],
//     dx/dv0 = -(1 - u - v) M^-1,  dx/dv1 = -u M^-1,  dx/dv2 = -v M^-1,
// so dLoss/dv_k = -w_k y with y = M^-T dLoss/dx = (g_t (e1 x e2) + g_u (d x e2) + g_v (e1 x d)) / a,
// a = e1 . (d x e2) being the Moeller-Trumbore determinant.  Vertex gradients are accumulated
// with atomicAdd through the face index map.
#include <cuda_runtime.h>

#include <algorithm>

#include "common.cuh"
#include "internal.hpp"
#include "persistent.cuh"
#include "variants.cuh"

namespace bvhgpu {

// Defined in kernels_trace.cu (same translation-unit-local helpers re-declared here).
namespace {

constexpr int kBlock = 128;
constexpr unsigned kFull = 0xFFFFFFFFu;
// The forward pass's long-ray schedule: a ray with more traversal steps than kLongSteps is served
// first by the next pass, spread evenly over the launch's warps.  Measured on the 512 x 512
// level-7 icosphere (median 21 steps, 99th percentile 395): 1.89 ms unscheduled; 1.64 ms at 250
// steps; 1.66 / 1.72 / 1.72 ms at 300 / 200 / 400; fixed caps of 1-4 long rays per warp instead of
// the even share 1.66-2.40 ms (long rays waiting for a free slot start late).
constexpr uint32_t kLongSteps = 250;

inline unsigned grid_for(uint32_t n, int block) { return (unsigned)((n + block - 1) / block); }

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

struct Shade {
    float3 d, lh, nh, n0, n1, n2, e1, e2;
    float ll, nl, c;
};

__device__ __forceinline__ float3 ld3(const float* p) { return make_float3(p[0], p[1], p[2]); }
__device__ __forceinline__ float3 sub3(float3 a, float3 b) { return make_float3(fsub(a.x, b.x), fsub(a.y, b.y), fsub(a.z, b.z)); }
__device__ __forceinline__ float3 add3(float3 a, float3 b) { return make_float3(fadd(a.x, b.x), fadd(a.y, b.y), fadd(a.z, b.z)); }
__device__ __forceinline__ float3 scale3(float3 a, float s) { return make_float3(fmul(a.x, s), fmul(a.y, s), fmul(a.z, s)); }
__device__ __forceinline__ float dotv(float3 a, float3 b) { return dot3(a.x, a.y, a.z, b.x, b.y, b.z); }
__device__ __forceinline__ float3 crossv(float3 a, float3 b) {
    return make_float3(fsub(fmul(a.y, b.z), fmul(a.z, b.y)), fsub(fmul(a.z, b.x), fmul(a.x, b.z)),
                       fsub(fmul(a.x, b.y), fmul(a.y, b.x)));
}

// Shading of a hit (t, u, v) on face f.  Returns the clamped intensity and the intermediates.
__device__ __forceinline__ float shade(float3 o, float3 d, float t, float u, float v, const uint32_t* faces,
                                       uint32_t f, const float* verts, const float* vnormals, float3 light,
                                       Shade& s) {
    const uint32_t i0 = faces[3ull * f], i1 = faces[3ull * f + 1], i2 = faces[3ull * f + 2];
    float3 p = add3(o, scale3(d, t));
    float3 l = sub3(light, p);
    s.ll = __fsqrt_rn(dotv(l, l));
    s.lh = make_float3(__fdiv_rn(l.x, s.ll), __fdiv_rn(l.y, s.ll), __fdiv_rn(l.z, s.ll));
    s.n0 = ld3(vnormals + 3ull * i0);
    s.n1 = ld3(vnormals + 3ull * i1);
    s.n2 = ld3(vnormals + 3ull * i2);
    float w0 = fsub(fsub(1.0f, u), v);
    float3 n = add3(add3(scale3(s.n0, w0), scale3(s.n1, u)), scale3(s.n2, v));
    s.nl = __fsqrt_rn(dotv(n, n));
    s.nh = make_float3(__fdiv_rn(n.x, s.nl), __fdiv_rn(n.y, s.nl), __fdiv_rn(n.z, s.nl));
    s.c = dotv(s.nh, s.lh);
    s.d = d;
    float3 v0 = ld3(verts + 3ull * i0);
    s.e1 = sub3(ld3(verts + 3ull * i1), v0);
    s.e2 = sub3(ld3(verts + 3ull * i2), v0);
    return s.c > 0.0f ? s.c : 0.0f;
}

__global__ void k_mesh_tris(const float* __restrict__ verts, const uint32_t* __restrict__ faces, uint32_t nf,
                            float4* __restrict__ tris, float4* __restrict__ tverts, float* __restrict__ pairs) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nf) return;
    const float* a = verts + 3ull * faces[3ull * i];
    const float* b = verts + 3ull * faces[3ull * i + 1];
    const float* c = verts + 3ull * faces[3ull * i + 2];
    float4 v0 = make_float4(a[0], a[1], a[2], 0.0f), v1 = make_float4(b[0], b[1], b[2], 0.0f),
           v2 = make_float4(c[0], c[1], c[2], 0.0f);
    float4 e1 = make_float4(fsub(v1.x, v0.x), fsub(v1.y, v0.y), fsub(v1.z, v0.z), 0.0f);
    float4 e2 = make_float4(fsub(v2.x, v0.x), fsub(v2.y, v0.y), fsub(v2.z, v0.z), 0.0f);
    tris[3ull * i] = v0;
    tris[3ull * i + 1] = e1;
    tris[3ull * i + 2] = e2;
    tverts[3ull * i] = v0;
    tverts[3ull * i + 1] = v1;
    tverts[3ull * i + 2] = v2;
    float comp[9] = {v0.x, v0.y, v0.z, e1.x, e1.y, e1.z, e2.x, e2.y, e2.z};
    float* P = pairs + 20ull * (i >> 1) + (i & 1u);
#pragma unroll
    for (int k = 0; k < 9; ++k) P[2 * k] = comp[k];
}

// Forward pass, persistent: each warp keeps 32 pixel slots and refills the finished ones from a
// global queue (ballot -> one atomicAdd per warp -> shfl), so that lanes whose pixel missed the
// mesh or finished early take new pixels instead of idling until the slowest ray of their block
// is done.  A finished pixel stores its hit record (the adjoint's checkpoint) and its intensity.
//
// Long rays (more than kLongSteps traversal steps: the silhouette's grazing rays, up to ~30x the
// median) sit side by side in pixel order, so a warp that draws a silhouette tile runs ~20 of them
// divergently together and the launch's tail is that warp.  With a schedule (`sched`, ForwardSchedule
// layout) each pass records its long rays, and the next pass serves them first from that list,
// an even share of them per warp at a time (any number once the pixel queue is empty), while
// the pixel queue skips them.  Every ray is traced exactly once either way:
// for i below the previous pass's ray count, flag_cur[i] is set exactly when i is in the list
// (the previous pass wrote both, for each of its rays), and each hit depends on its ray only.
template <int BLOCK, int MINB, class STK>
__global__ void __launch_bounds__(BLOCK, MINB) k_lambert_forward(GBlas b, const float4* __restrict__ rays, uint32_t n,
                                                                 const uint32_t* __restrict__ faces,
                                                                 const float* __restrict__ verts,
                                                                 const float* __restrict__ vnormals, float3 light,
                                                                 float* __restrict__ image, GHit* __restrict__ hits,
                                                                 uint32_t* queue, uint32_t* sched, uint32_t cap,
                                                                 LeafPolicy pol, uint32_t refill, uint32_t* err) {
    extern __shared__ uint2 stack_smem[];
    const unsigned lane = threadIdx.x & 31u;
    int phase = 0;  // 0 needs a pixel, 1 tracing, 3 retired
    uint32_t idx = 0;
    LaneRay r;
    TravT<STK> tr;
    tr.stk.bind(stack_smem);
    StepResult st = kStepFinished;
    bool queue_open = true;
    // the schedule of this pass (pass number k): the previous pass's flags and list (parity k & 1),
    // its ray count, and the flags and list this pass writes for the next one
    uint32_t parity = 0, lcount = 0, n_prev = 0;
    const uint32_t* flag_cur = nullptr;
    const uint32_t* list_cur = nullptr;
    uint32_t* flag_nxt = nullptr;
    uint32_t* list_nxt = nullptr;
    uint32_t* ctr = nullptr;
    if (sched != nullptr) {
        ctr = sched + ForwardSchedule::counters(cap);
        queue = ctr + ForwardSchedule::kQueue;
        parity = *reinterpret_cast<volatile uint32_t*>(ctr + ForwardSchedule::kPass) & 1u;
        n_prev = *reinterpret_cast<volatile uint32_t*>(ctr + ForwardSchedule::kPrevRays);
        flag_cur = sched + ForwardSchedule::flags(cap, parity);
        list_cur = sched + ForwardSchedule::list(cap, parity);
        flag_nxt = sched + ForwardSchedule::flags(cap, parity ^ 1u);
        list_nxt = sched + ForwardSchedule::list(cap, parity ^ 1u);
        lcount = min(*reinterpret_cast<volatile uint32_t*>(ctr + ForwardSchedule::kCount + parity), cap);
    }
    bool long_open = lcount > 0u;
    bool is_long = false;
    Deadline dl;
    dl.start(err);
    for (;;) {
        if (dl.expired(err)) {
            if (ctr != nullptr && lane == 0u) atomicExch(ctr + ForwardSchedule::kStopped, 1u);
            return;
        }
        const unsigned need = __ballot_sync(kFull, phase == 0);
        const unsigned busy = __ballot_sync(kFull, phase == 1);
        const unsigned longs = __ballot_sync(kFull, phase == 1 && is_long);
        // refill once `refill` lanes are idle (or none is busy)
        if (need != 0u && ((uint32_t)__popc(need) >= refill || busy == 0u)) {
            const int leader = __ffs(need) - 1;
            const uint32_t nn = (uint32_t)__popc(need);
            const uint32_t rank = (uint32_t)__popc(need & ((1u << lane) - 1u));
            // the previous pass's long rays first
            uint32_t want = 0, got = 0, lb = 0;
            if (long_open) {
                const uint32_t act = (uint32_t)__popc(longs);
                const uint32_t warps = gridDim.x * (BLOCK / 32);
                const uint32_t share = max(1u, (lcount + warps - 1u) / warps);
                want = !queue_open ? nn : act < share ? min(nn, share - act) : 0u;
                if (want) {
                    if ((int)lane == leader) lb = atomicAdd(ctr + ForwardSchedule::kHead, want);
                    lb = __shfl_sync(kFull, lb, leader);
                    got = lb >= lcount ? 0u : min(want, lcount - lb);
                    if (lb + want >= lcount) long_open = false;
                }
            }
            const uint32_t nreg = queue_open ? nn - got : 0u;
            uint32_t base = 0;
            if (nreg) {
                if ((int)lane == leader) base = atomicAdd(queue, nreg);
                base = __shfl_sync(kFull, base, leader);
                if (base + nreg >= n) queue_open = false;
            }
            if (phase == 0) {
                uint32_t my = n;
                if (rank < got) {
                    my = __ldcg(list_cur + lb + rank);  // an entry >= n (a larger previous pass) is skipped
                    is_long = true;
                } else if (nreg) {
                    my = base + rank - got;
                    if (my < n_prev && __ldcg(flag_cur + my) != 0u) my = n;  // in the list
                    is_long = false;
                }
                if (my < n) {
                    idx = my;
                    float3 o, d;
                    float t0;
                    load_ray(rays, idx, o, d, t0);
                    init_lane_ray(r, o, d, t0);
                    tr.init(b);
                    st = kStepContinue;
                    phase = 1;
                } else if (!queue_open && !long_open) {
                    phase = 3;
                }
            }
        }
        if (phase == 1) {
            if (st == kStepContinue) st = tr.advance(b, r, pol, err);
            if (st == kStepFinished) {
                const bool hit = r.hit && r.ct < FLT_MAX;
                store_hit(hits, idx, hit, r.ct, r.hu, r.hv, r.hp, 0u);
                float I = 0.0f;
                if (hit) {
                    Shade sh;
                    I = shade(r.o, r.d, r.ct, r.hu, r.hv, faces, r.hp, verts, vnormals, light, sh);
                }
                image[idx] = I;
                if (sched != nullptr) {
                    const bool lng = tr.steps > kLongSteps;
                    __stcg(flag_nxt + idx, lng ? 1u : 0u);
                    if (lng) {
                        const uint32_t slot = atomicAdd(ctr + ForwardSchedule::kCount + (parity ^ 1u), 1u);
                        if (slot < cap) __stcg(list_nxt + slot, idx);  // a ray finishes once a pass: always true
                    }
                }
                phase = 0;
            }
        }
        const unsigned pend = __ballot_sync(kFull, phase == 1 && st == kStepBigLeaf);
        if (pend == 0u) {
            if (!queue_open && !long_open && __ballot_sync(kFull, phase == 0 || phase == 1) == 0u) break;
            continue;
        }
        coop_leaf_phase(pend, b, tr, r, st);
    }
}

// Starts a scheduled forward pass over n rays: the next pass number (its parity alternates, also
// across the counter's wrap), the previous pass's ray count (0, and an empty list, when that pass
// stopped at a deadline), empty queues, and an empty list for the pass after it.
__global__ void k_forward_prep(uint32_t* ctr, uint32_t n) {
    const uint32_t k = ctr[ForwardSchedule::kPass] + 1u;
    const bool stopped = ctr[ForwardSchedule::kStopped] != 0u;
    ctr[ForwardSchedule::kPass] = k;
    ctr[ForwardSchedule::kPrevRays] = stopped ? 0u : ctr[ForwardSchedule::kRays];
    ctr[ForwardSchedule::kRays] = n;
    ctr[ForwardSchedule::kStopped] = 0u;
    if (stopped) ctr[ForwardSchedule::kCount + (k & 1u)] = 0u;
    ctr[ForwardSchedule::kQueue] = 0u;
    ctr[ForwardSchedule::kHead] = 0u;
    ctr[ForwardSchedule::kCount + ((k & 1u) ^ 1u)] = 0u;
}

// Per-block partial sums of (I - T)^2 in double.
__global__ void k_mse_partials(const float* __restrict__ image, const float* __restrict__ target, uint32_t n,
                               double* __restrict__ partials) {
    __shared__ double sh[256];
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    double v = 0.0;
    if (i < n) {
        double e = (double)image[i] - (double)target[i];
        v = e * e;
    }
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) partials[blockIdx.x] = sh[0];
}

__global__ void __launch_bounds__(kBlock) k_lambert_adjoint(const float4* __restrict__ rays, uint32_t n,
                                                            const GHit* __restrict__ hits,
                                                            const float* __restrict__ image,
                                                            const float* __restrict__ target,
                                                            const uint32_t* __restrict__ faces,
                                                            const float* __restrict__ verts,
                                                            const float* __restrict__ vnormals, float3 light,
                                                            float scale, float* __restrict__ grad) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const GHit h = hits[i];
    if (h.prim == kMiss) return;
    float3 o, d;
    float t0;
    load_ray(rays, i, o, d, t0);
    Shade s;
    float I = shade(o, d, h.t, h.u, h.v, faces, h.prim, verts, vnormals, light, s);
    if (!(s.c > 0.0f)) return;  // max(0, .) is flat there
    const float g = fmul(scale, fsub(image[i], target[i]));  // dLoss/dI of the mean squared error
    (void)I;
    // dI/dn = (lh - c nh) / |n|,  dI/dl = (nh - c lh) / |l|
    float3 dn = scale3(sub3(s.lh, scale3(s.nh, s.c)), __frcp_rn(s.nl));
    float3 dl = scale3(sub3(s.nh, scale3(s.lh, s.c)), __frcp_rn(s.ll));
    const float gt = fmul(g, -dotv(dl, d));                 // l = L - o - t d
    const float gu = fmul(g, dotv(dn, sub3(s.n1, s.n0)));
    const float gv = fmul(g, dotv(dn, sub3(s.n2, s.n0)));
    const float a = dotv(s.e1, crossv(d, s.e2));
    const float f = __frcp_rn(a);
    float3 y = add3(add3(scale3(crossv(s.e1, s.e2), gt), scale3(crossv(d, s.e2), gu)), scale3(crossv(s.e1, d), gv));
    y = scale3(y, f);
    const float w[3] = {fsub(fsub(1.0f, h.u), h.v), h.u, h.v};
    for (int k = 0; k < 3; ++k) {
        const uint32_t vid = faces[3ull * h.prim + k];
        const float m = -w[k];
        atomicAdd(grad + 3ull * vid, fmul(m, y.x));
        atomicAdd(grad + 3ull * vid + 1, fmul(m, y.y));
        atomicAdd(grad + 3ull * vid + 2, fmul(m, y.z));
    }
}

__global__ void k_sgd(float* __restrict__ verts, float* __restrict__ grad, uint32_t count, float lr) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    verts[i] = fsub(verts[i], fmul(lr, grad[i]));
    grad[i] = 0.0f;
}

}  // namespace

cudaError_t launch_mesh_update(bvhgpu_ctx* ctx, DeviceMesh& m, DeviceBlas& b, cudaStream_t s) {
    {
        LaunchScope scope(ctx, BVHGPU_K_OTHER, s);
        k_mesh_tris<<<grid_for(m.nfaces, 256), 256, 0, s>>>(m.verts, m.faces, m.nfaces, b.tris, b.verts,
                                                            reinterpret_cast<float*>(b.pairs));
        g_launches++;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if ((e = launch_hidden_refresh(ctx, b, s)) != cudaSuccess) return e;
    return launch_refit(ctx, b, s);
}

cudaError_t launch_lambert_forward(bvhgpu_ctx* ctx, DeviceMesh& m, const DeviceBlas& b, const float4* rays, uint32_t n,
                                   const float* light, float* image, void* hits, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    GBlas g = to_gblas(b);
    float3 L = make_float3(light[0], light[1], light[2]);
    // the launch shape, stack and leaf policy (big leaves, hidden-tree margin) of the plain trace
    // kernel's launch config, and its refill threshold
    const Variant v = resolve(ctx->tune[BVHGPU_K_TRACE_BLAS], b.depth);
    uint32_t* queue = ctx->d_scratch + 5;
    cudaError_t e = cudaSuccess;
    // the long-ray schedule (ForwardSchedule): grown outside stream capture only; a captured pass
    // that finds it too small runs in pixel order (its results are the same)
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if ((e = cudaStreamIsCapturing(s, &cs)) != cudaSuccess) return e;
    if (m.sched_cap < n && cs == cudaStreamCaptureStatusNone) {
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
        cudaFree(m.sched);
        m.sched = nullptr;
        m.sched_cap = 0;
        const size_t bytes = 4ull * ForwardSchedule::words(n);
        if ((e = cudaMalloc(&m.sched, bytes)) != cudaSuccess) return e;
        if ((e = cudaMemsetAsync(m.sched, 0, bytes, s)) != cudaSuccess) return e;
        m.sched_cap = n;
    }
    uint32_t* sched = m.sched_cap >= n ? m.sched : nullptr;
    if (sched != nullptr) {
        k_forward_prep<<<1, 1, 0, s>>>(sched + ForwardSchedule::counters(m.sched_cap), n);
        g_launches++;
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    } else if ((e = cudaMemsetAsync(queue, 0, sizeof(uint32_t), s)) != cudaSuccess) {
        return e;
    }
    LaunchScope scope(ctx, BVHGPU_K_LAMBERT_FORWARD, s);
    e = with_variant(v.shape, v.stack, [&](auto sh, auto tg) {
        using SH = decltype(sh);
        using STK = typename decltype(tg)::type;
        auto* k = k_lambert_forward<SH::block, SH::minb, STK>;
        const size_t smem = stack_smem_bytes<STK>(SH::block);
        k<<<persistent_grid(ctx, k, SH::block, smem), SH::block, smem, s>>>(
            g, rays, n, m.faces, m.verts, m.vnormals, L, image, static_cast<GHit*>(hits), queue, sched, m.sched_cap,
            v.pol, v.refill, ctx->d_err);
        return cudaGetLastError();
    });
    g_launches++;
    return e;
}

cudaError_t launch_mse_partials(bvhgpu_ctx* ctx, const float* image, const float* target, uint32_t n, double* partials,
                                cudaStream_t s) {
    LaunchScope scope(ctx, BVHGPU_K_OTHER, s);
    k_mse_partials<<<grid_for(n, 256), 256, 0, s>>>(image, target, n, partials);
    g_launches++;
    return cudaGetLastError();
}

cudaError_t launch_lambert_adjoint(bvhgpu_ctx* ctx, DeviceMesh& m, const float4* rays, uint32_t n, const float* light,
                                   const void* hits, const float* image, const float* target, float* grad,
                                   cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    float3 L = make_float3(light[0], light[1], light[2]);
    LaunchScope scope(ctx, BVHGPU_K_LAMBERT_ADJOINT, s);
    k_lambert_adjoint<<<grid_for(n, kBlock), kBlock, 0, s>>>(rays, n, static_cast<const GHit*>(hits), image, target,
                                                             m.faces, m.verts, m.vnormals, L, 2.0f / (float)n, grad);
    g_launches++;
    return cudaGetLastError();
}

cudaError_t launch_sgd(bvhgpu_ctx* ctx, DeviceMesh& m, float* grad, float lr, cudaStream_t s) {
    LaunchScope scope(ctx, BVHGPU_K_OTHER, s);
    k_sgd<<<grid_for(3 * m.nverts, 256), 256, 0, s>>>(m.verts, grad, 3 * m.nverts, lr);
    g_launches++;
    return cudaGetLastError();
}

}  // namespace bvhgpu
