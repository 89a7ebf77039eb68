// Launch configurations of the traversal kernels and the autotuner.
//
// The tuner times a caller-supplied job (one of the library's own async calls) under candidate
// configs: a coordinate search from the current config, one dimension at a time (launch shape,
// stack, big-leaf threshold, refill, hidden-tree margin), two sweeps, each candidate timed by events on the context
// stream after an untimed run.  Configs never change results, only speed, so the job may be the
// caller's real workload.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <map>
#include <tuple>
#include <vector>

#include "internal.hpp"
#include "variants.cuh"

using namespace bvhgpu;

namespace {

constexpr uint32_t kBigLeafValues[] = {8u, 16u, 32u, 64u, BVHGPU_BIG_LEAF_NEVER};
constexpr uint32_t kRefillValues[] = {1u, 8u, 16u};
constexpr uint32_t kHiddenValues[] = {0u, 100u, 250u, 500u, 1000u};

bool tunable(int k) {
    return k == BVHGPU_K_TRACE_BLAS || k == BVHGPU_K_TRACE_SCENE || k == BVHGPU_K_PERSISTENT_BOUNCE ||
           k == BVHGPU_K_TRACE_BATCH || k == BVHGPU_K_SCENE_BOUNCE;
}

bool persistent(int k) {
    return k == BVHGPU_K_PERSISTENT_BOUNCE || k == BVHGPU_K_TRACE_BATCH || k == BVHGPU_K_SCENE_BOUNCE;
}

bool valid_config(const bvhgpu_tune_config& c) {
    if (shape_index(c.block, c.min_blocks) < 0) return false;
    if (c.stack != 0 && c.stack != 8 && c.stack != 32 && c.stack != 256) return false;
    return c.refill >= 1u && c.refill <= 32u && c.hidden <= 1000000u;
}

int run_job(bvhgpu_ctx* ctx, const bvhgpu_tune_job& j) {
    switch (j.kernel) {
        case BVHGPU_K_TRACE_BLAS:
            if (j.nitems)
                return bvhgpu_trace_batch_async(ctx, j.items, j.nitems, j.d_rays, j.n, BVHGPU_MODE_PLAIN, j.d_hits0,
                                                nullptr);
            return bvhgpu_blas_intersect_async(ctx, j.target, j.d_rays, j.n, j.d_hits0, nullptr);
        case BVHGPU_K_PERSISTENT_BOUNCE:
            return bvhgpu_blas_trace_bounce_async(ctx, j.target, j.d_rays, j.n, j.seed, BVHGPU_MODE_PERSISTENT,
                                                  j.d_hits0, j.d_hits1, nullptr);
        case BVHGPU_K_TRACE_SCENE:
            return bvhgpu_scene_intersect_async(ctx, j.target, j.d_rays, j.n, j.d_hits0, nullptr);
        case BVHGPU_K_SCENE_BOUNCE:
            return bvhgpu_scene_trace_bounce_async(ctx, j.target, j.d_rays, j.n, j.seed, j.d_hits0, j.d_hits1,
                                                   nullptr);
        case BVHGPU_K_TRACE_BATCH:
            return bvhgpu_trace_batch_async(ctx, j.items, j.nitems, j.d_rays, j.n, BVHGPU_MODE_PERSISTENT, j.d_hits0,
                                            nullptr);
        default:
            return BVHGPU_ERR_INVALID_ARG;
    }
}

// Depth of the deepest tree the job traverses (stacks below it resolve to the same variant).
uint32_t job_depth(bvhgpu_ctx* ctx, const bvhgpu_tune_job& j) {
    uint32_t d = 1;
    auto blas_depth = [&](uint32_t id) {
        auto it = ctx->blas.find(id);
        if (it != ctx->blas.end()) d = std::max(d, it->second.depth);
    };
    if (j.nitems) {
        for (uint32_t i = 0; i < j.nitems; ++i) blas_depth(j.items[i].blas);
    } else if (j.kernel == BVHGPU_K_TRACE_SCENE || j.kernel == BVHGPU_K_SCENE_BOUNCE) {
        auto it = ctx->scenes.find(j.target);
        if (it != ctx->scenes.end())
            for (uint32_t id : it->second.table_blas) blas_depth(id);
    } else {
        blas_depth(j.target);
    }
    return d;
}

struct Timer {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    Timer() {
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
    }
    ~Timer() {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }
};

// Median ms per call of the job under cfg, or a negative value if a call failed.
float measure(bvhgpu_ctx* ctx, const bvhgpu_tune_job& j, const bvhgpu_tune_config& cfg, uint32_t reps, Timer& tm) {
    ctx->tune[j.kernel] = cfg;
    if (run_job(ctx, j) != BVHGPU_OK || bvhgpu_sync(ctx) != BVHGPU_OK) return -1.0f;
    std::vector<float> ms;
    for (uint32_t r = 0; r < reps; ++r) {
        cudaEventRecord(tm.e0, ctx->stream);
        if (run_job(ctx, j) != BVHGPU_OK) return -1.0f;
        cudaEventRecord(tm.e1, ctx->stream);
        if (cudaEventSynchronize(tm.e1) != cudaSuccess) return -1.0f;
        float t = 0.0f;
        cudaEventElapsedTime(&t, tm.e0, tm.e1);
        ms.push_back(t);
    }
    if (bvhgpu_sync(ctx) != BVHGPU_OK) return -1.0f;
    std::sort(ms.begin(), ms.end());
    return ms[ms.size() / 2];
}

}  // namespace

extern "C" {

int bvhgpu_tune_get(bvhgpu_ctx* ctx, int kernel, bvhgpu_tune_config* out) {
    if (!ctx || !out || !tunable(kernel)) return BVHGPU_ERR_INVALID_ARG;
    *out = ctx->tune[kernel];
    return BVHGPU_OK;
}

int bvhgpu_tune_set(bvhgpu_ctx* ctx, int kernel, const bvhgpu_tune_config* cfg) {
    if (!ctx || !cfg) return BVHGPU_ERR_INVALID_ARG;
    if (!tunable(kernel)) return record_error(ctx, BVHGPU_ERR_INVALID_ARG, "tune_set: kernel has no variants");
    if (!valid_config(*cfg)) return record_error(ctx, BVHGPU_ERR_INVALID_ARG, "tune_set: variant not compiled");
    ctx->tune[kernel] = *cfg;
    return BVHGPU_OK;
}

int bvhgpu_tune_space(int kernel, bvhgpu_tune_config* out, uint32_t cap, uint32_t* count) {
    if (!tunable(kernel) || (cap && !out)) return BVHGPU_ERR_INVALID_ARG;
    const uint32_t nrefill = persistent(kernel) ? 3u : 1u;
    uint32_t k = 0;
    for (int sh = 0; sh < kNumShapes; ++sh)
        for (int st = 0; st < kNumStacks; ++st)
            for (uint32_t bl : kBigLeafValues)
                for (uint32_t rf = 0; rf < nrefill; ++rf)
                    for (uint32_t hd : kHiddenValues) {
                        if (k < cap)
                            out[k] = bvhgpu_tune_config{(uint32_t)kShapeBlock[sh], (uint32_t)kShapeMinBlocks[sh],
                                                        (uint32_t)kStackSizes[st], bl, kRefillValues[rf], hd};
                        ++k;
                    }
    if (count) *count = k;
    return BVHGPU_OK;
}

int bvhgpu_autotune(bvhgpu_ctx* ctx, const bvhgpu_tune_job* job, uint32_t reps, bvhgpu_tune_config* best,
                    float* best_ms) {
    if (!ctx || !job) return BVHGPU_ERR_INVALID_ARG;
    if (!tunable(job->kernel)) return record_error(ctx, BVHGPU_ERR_INVALID_ARG, "autotune: kernel has no variants");
    if (ctx->capturing) return record_error(ctx, BVHGPU_ERR_INVALID_ARG, "autotune: not allowed during capture");
    if (reps == 0) reps = 1;
    const bvhgpu_tune_job j = *job;
    const uint32_t depth = job_depth(ctx, j);
    Timer tm;
    // measured configs, keyed by the variant they resolve to plus the run-time knobs
    std::map<std::tuple<int, int, uint32_t, uint32_t, uint32_t>, float> seen;
    auto key = [&](const bvhgpu_tune_config& c) {
        const Variant v = resolve(c, depth);
        return std::make_tuple(v.shape, v.stack, v.pol.big_leaf, persistent(j.kernel) ? v.refill : 1u, c.hidden);
    };
    auto time_of = [&](const bvhgpu_tune_config& c) -> float {
        auto k = key(c);
        auto it = seen.find(k);
        if (it != seen.end()) return it->second;
        float ms = measure(ctx, j, c, reps, tm);
        if (ms < 0.0f) ms = 3.4e38f;  // a failed candidate (e.g. not launchable) never wins
        seen[k] = ms;
        return ms;
    };
    bvhgpu_tune_config cur = ctx->tune[j.kernel];
    if (!valid_config(cur)) cur = bvhgpu_tune_config{128u, 5u, 256u, 16u, 8u, 500u};
    float cur_ms = time_of(cur);
    auto consider = [&](const bvhgpu_tune_config& c) {
        const float ms = time_of(c);
        if (ms < 0.99f * cur_ms) {  // 1 % margin against timing noise
            cur = c;
            cur_ms = ms;
        }
    };
    for (int sweep = 0; sweep < 2; ++sweep) {
        const bvhgpu_tune_config base_shape = cur;
        for (int sh = 0; sh < kNumShapes; ++sh) {
            bvhgpu_tune_config c = base_shape;
            c.block = (uint32_t)kShapeBlock[sh];
            c.min_blocks = (uint32_t)kShapeMinBlocks[sh];
            consider(c);
        }
        const bvhgpu_tune_config base_stack = cur;
        for (int st = 0; st < kNumStacks; ++st) {
            bvhgpu_tune_config c = base_stack;
            c.stack = (uint32_t)kStackSizes[st];
            consider(c);
        }
        const bvhgpu_tune_config base_leaf = cur;
        for (uint32_t bl : kBigLeafValues) {
            bvhgpu_tune_config c = base_leaf;
            c.big_leaf = bl;
            consider(c);
        }
        const bvhgpu_tune_config base_hidden = cur;
        for (uint32_t hd : kHiddenValues) {
            bvhgpu_tune_config c = base_hidden;
            c.hidden = hd;
            consider(c);
        }
        if (persistent(j.kernel)) {
            const bvhgpu_tune_config base_refill = cur;
            for (uint32_t rf : kRefillValues) {
                bvhgpu_tune_config c = base_refill;
                c.refill = rf;
                consider(c);
            }
        }
    }
    ctx->tune[j.kernel] = cur;
    if (cur_ms >= 3.0e38f) return record_error(ctx, BVHGPU_ERR_CUDA, "autotune: no candidate ran");
    if (best) *best = cur;
    if (best_ms) *best_ms = cur_ms;
    return BVHGPU_OK;
}

}  // extern "C"
