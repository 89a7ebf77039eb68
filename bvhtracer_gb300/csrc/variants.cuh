// Compiled variants of the traversal kernels, picked per launch from a bvhgpu_tune_config.
//
// A variant is (block size, register budget, stack):
//  - the launch shape: threads per block and the minimum blocks per SM handed to
//    __launch_bounds__, which caps registers per thread (65,536 / (block * min_blocks));
//  - the stack: 8 or 32 entries (4 in registers, the rest in shared memory), or 256 entries in
//    local memory for deep trees.
// The run-time knobs (leaf policy: big-leaf threshold and hidden-tree margin; refill) are kernel
// arguments.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

#include "../../include/bvhgpu.h"
#include "common.cuh"

namespace bvhgpu {

template <int B, int M>
struct Shape {
    static constexpr int block = B;
    static constexpr int minb = M;
};

template <class T>
struct Tag {
    using type = T;
};

using StackS8 = SplitStack<4, 4>;
using StackS32 = SplitStack<4, 28>;
using StackL256 = LocalStack<256>;

constexpr int kNumShapes = 5;
constexpr int kShapeBlock[kNumShapes] = {128, 128, 128, 128, 64};
constexpr int kShapeMinBlocks[kNumShapes] = {1, 5, 6, 8, 1};
constexpr int kNumStacks = 3;
constexpr int kStackSizes[kNumStacks] = {8, 32, 256};

template <class STK>
constexpr size_t stack_smem_bytes(int block) {
    return (size_t)STK::kSharedEntries * sizeof(uint2) * (size_t)block;
}

template <class SH, class F>
decltype(auto) with_stack(int stack, F&& f) {
    switch (stack) {
        case 8: return f(SH{}, Tag<StackS8>{});
        case 32: return f(SH{}, Tag<StackS32>{});
        default: return f(SH{}, Tag<StackL256>{});
    }
}

// Calls f(Shape<...>{}, Tag<Stack>{}) for the variant (shape index, stack entries).
template <class F>
decltype(auto) with_variant(int shape, int stack, F&& f) {
    switch (shape) {
        case 1: return with_stack<Shape<128, 5>>(stack, f);
        case 2: return with_stack<Shape<128, 6>>(stack, f);
        case 3: return with_stack<Shape<128, 8>>(stack, f);
        case 4: return with_stack<Shape<64, 1>>(stack, f);
        default: return with_stack<Shape<128, 1>>(stack, f);
    }
}

// A tune config resolved against one launch: shape index, stack entries, run-time knobs.
struct Variant {
    int shape;
    int stack;
    LeafPolicy pol;
    uint32_t refill;
};

// Smallest compiled stack holding `depth - 1` pending far children.
inline int min_stack_for_depth(uint32_t depth) {
    for (int k = 0; k < kNumStacks; ++k)
        if ((uint32_t)kStackSizes[k] + 1u >= depth) return kStackSizes[k];
    return kStackSizes[kNumStacks - 1];
}

inline int shape_index(uint32_t block, uint32_t min_blocks) {
    for (int k = 0; k < kNumShapes; ++k)
        if ((uint32_t)kShapeBlock[k] == block && (uint32_t)kShapeMinBlocks[k] == min_blocks) return k;
    return -1;
}

// The config as it applies to a tree of `depth`: a stack too small for it (or 0) becomes the
// smallest that holds it, so a tuned config never fails on a deeper tree.
inline Variant resolve(const bvhgpu_tune_config& c, uint32_t depth) {
    Variant v;
    v.shape = shape_index(c.block, c.min_blocks);
    if (v.shape < 0) v.shape = 0;
    const int need = min_stack_for_depth(depth);
    const int want = (int)c.stack > need ? (int)c.stack : need;
    v.stack = kStackSizes[kNumStacks - 1];
    for (int k = kNumStacks - 1; k >= 0; --k)
        if (kStackSizes[k] >= want) v.stack = kStackSizes[k];
    v.pol.big_leaf = c.big_leaf;
    v.pol.max_duv = (float)c.hidden * 1e-3f;
    v.refill = c.refill < 1u ? 1u : (c.refill > 32u ? 32u : c.refill);
    return v;
}

}  // namespace bvhgpu
