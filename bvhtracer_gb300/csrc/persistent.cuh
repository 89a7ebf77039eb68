// Pieces shared by the warp-synchronous and persistent traversal kernels: lane ray setup, the
// warp-cooperative big-leaf phase, and the grid of a persistent launch.
#pragma once

#include <cuda_runtime.h>

#include "common.cuh"
#include "internal.hpp"

namespace bvhgpu {

__device__ __forceinline__ void init_lane_ray(LaneRay& r, float3 o, float3 d, float t) {
    r.o = o;
    r.d = d;
    r.rd = recip3(d);
    r.ct = t;
    r.hu = r.hv = 0.0f;
    r.hp = 0;
    r.hit = false;
}

// Cooperative leaf phase: lanes waiting on the same leaf form a group; the group's rays are
// tested two at a time (coop_leaf2 shares each loaded triangle pair between the two rays), an
// odd one alone; with QUAD, four at a time when four share their origin (coop_leaf4).  QUAD is on
// where in-order leaves dominate -- the batch kernel and the plain per-scene kernel (16 of the
// uneven batch's scenes: 88.5 -> 81.6 ms and 106.6 -> 94.8 ms; the plain icosphere frame 1 % slower)
// -- and off in the headline and instanced kernels, which lost 3.5 % and 30 % to its registers.
// `key` identifies the BLAS (pairs pointer) so that different scenes of a batch never share a leaf.
template <bool QUAD = false, class TR>
__device__ __forceinline__ void coop_leaf_phase(unsigned pend, const GBlas& blas, TR& tr, LaneRay& r, StepResult& st) {
    const unsigned lane = threadIdx.x & 31u;
    const unsigned long long key = reinterpret_cast<unsigned long long>(blas.pairs);
    while (pend) {
        const int leader = __ffs(pend) - 1;
        const uint32_t f = __shfl_sync(0xFFFFFFFFu, tr.first, leader);
        const uint32_t c = __shfl_sync(0xFFFFFFFFu, tr.cnt, leader);
        const unsigned long long lk = __shfl_sync(0xFFFFFFFFu, key, leader);
        const ulonglong2* P = reinterpret_cast<const ulonglong2*>(lk);
        unsigned group = __ballot_sync(0xFFFFFFFFu, ((pend >> lane) & 1u) && tr.first == f && key == lk);
        pend &= ~group;
        while (group) {
            if (QUAD && __popc(group) >= 4) {
                // four rays at once when they share their origin (primaries of one camera)
                unsigned g = group;
                const int q0 = __ffs(g) - 1;
                g &= g - 1u;
                const int q1 = __ffs(g) - 1;
                g &= g - 1u;
                const int q2 = __ffs(g) - 1;
                g &= g - 1u;
                const int q3 = __ffs(g) - 1;
                const unsigned ox = __float_as_uint(r.o.x), oy = __float_as_uint(r.o.y), oz = __float_as_uint(r.o.z);
                const bool same = __shfl_sync(0xFFFFFFFFu, ox, q0) == __shfl_sync(0xFFFFFFFFu, ox, q1) &&
                                  __shfl_sync(0xFFFFFFFFu, ox, q0) == __shfl_sync(0xFFFFFFFFu, ox, q2) &&
                                  __shfl_sync(0xFFFFFFFFu, ox, q0) == __shfl_sync(0xFFFFFFFFu, ox, q3) &&
                                  __shfl_sync(0xFFFFFFFFu, oy, q0) == __shfl_sync(0xFFFFFFFFu, oy, q1) &&
                                  __shfl_sync(0xFFFFFFFFu, oy, q0) == __shfl_sync(0xFFFFFFFFu, oy, q2) &&
                                  __shfl_sync(0xFFFFFFFFu, oy, q0) == __shfl_sync(0xFFFFFFFFu, oy, q3) &&
                                  __shfl_sync(0xFFFFFFFFu, oz, q0) == __shfl_sync(0xFFFFFFFFu, oz, q1) &&
                                  __shfl_sync(0xFFFFFFFFu, oz, q0) == __shfl_sync(0xFFFFFFFFu, oz, q2) &&
                                  __shfl_sync(0xFFFFFFFFu, oz, q0) == __shfl_sync(0xFFFFFFFFu, oz, q3);
                if (same) {
                    group = g & (g - 1u);
                    coop_leaf4(P, f, c, q0, q1, q2, q3, r);
                    if ((int)lane == q0 || (int)lane == q1 || (int)lane == q2 || (int)lane == q3) {
                        if constexpr (TR::kCount) tr.cn.coop_tris += c;
                        st = tr.pop() ? kStepFinished : kStepContinue;
                    }
                    continue;
                }
            }
            const int a = __ffs(group) - 1;
            group &= group - 1u;
            if (group) {
                const int b = __ffs(group) - 1;
                group &= group - 1u;
                coop_leaf2(P, f, c, a, b, r);
                if ((int)lane == a || (int)lane == b) {
                    if constexpr (TR::kCount) tr.cn.coop_tris += c;
                    st = tr.pop() ? kStepFinished : kStepContinue;
                }
            } else {
                coop_leaf(P, f, c, a, r);
                if ((int)lane == a) {
                    if constexpr (TR::kCount) tr.cn.coop_tris += c;
                    st = tr.pop() ? kStepFinished : kStepContinue;
                }
            }
        }
    }
}

// Blocks of a persistent launch: as many as fit on all SMs at once.
template <class K>
int persistent_grid(bvhgpu_ctx* ctx, K kernel, int block, size_t smem) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem);
    if (per_sm < 1) per_sm = 1;
    return per_sm * ctx->num_sms;
}

}  // namespace bvhgpu
