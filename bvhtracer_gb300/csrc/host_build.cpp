// Host SAH binned BVH build: the reference's BvhBuilder::build_for (BT/src/model/bvh.rs:317-541),
// producing the same node array and the same triangle order, bit for bit.
//
// Differences in structure only (none in results): centroids are computed once per triangle
// (the reference recomputes Triangle::centroid, triangle.rs:33-39, with the same f32 ops each
// time) and permuted with the triangles; the recursion (bvh.rs:465-466) becomes an explicit
// LIFO work list that pops the left child first, which allocates nodes in the same
// depth-first order; the three axes are binned in one pass over the node's triangles.
//
// Compiled with -ffp-contract=off: no multiply-add is fused, as in Rust.

#include <cfloat>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>

#include "internal.hpp"

namespace bvhgpu {
namespace {

// f32::min / f32::max semantics: a NaN operand is ignored; on equality the first operand
// is kept (Rust leaves the sign of a zero result unspecified).
inline float min_nan_ignoring(float a, float b) {
    if (a != a) return b;
    if (b != b) return a;
    return (b < a) ? b : a;
}
inline float max_nan_ignoring(float a, float b) {
    if (a != a) return b;
    if (b != b) return a;
    return (b > a) ? b : a;
}

struct Box {
    float lo[3];
    float hi[3];
};

inline void box_zero(Box& b) { std::memset(&b, 0, sizeof(b)); }  // Aabb::default (aabb.rs:11-19)
inline void box_grow(Box& b, const float* p) {                     // Aabb::grow (aabb.rs:36-39)
    for (int k = 0; k < 3; ++k) {
        b.lo[k] = min_nan_ignoring(b.lo[k], p[k]);
        b.hi[k] = max_nan_ignoring(b.hi[k], p[k]);
    }
}
inline float box_area(const Box& b) {  // Aabb::area (aabb.rs:48-57)
    float ex = b.hi[0] - b.lo[0];
    float ey = b.hi[1] - b.lo[1];
    float ez = b.hi[2] - b.lo[2];
    return ex * ey + ey * ez + ez * ex;
}

// Rust `f as usize`: saturating conversion, NaN -> 0.
inline uint64_t f32_to_usize(float f) {
    if (!(f > 0.0f)) return 0;
    if (f >= 18446744073709551616.0f) return UINT64_MAX;
    return (uint64_t)f;
}

struct Builder {
    float* tris;       // n x 9, permuted in place
    uint32_t* perm = nullptr;  // optional: original index of the triangle at each position
    uint32_t n;
    std::vector<float> cent;  // n x 3
    bvhgpu_node* nodes;
    uint32_t nodes_used = 2;

    void compute_centroids() {
        const float one = 1.0f;
        const float third = one / (one + one + one);
        cent.resize(3ull * n);
        for (uint32_t i = 0; i < n; ++i) {
            const float* t = tris + 9ull * i;
            for (int k = 0; k < 3; ++k) cent[3ull * i + k] = ((t[k] + t[3 + k]) + t[6 + k]) * third;
        }
    }

    // update_node_bounds (bvh.rs:317-330): start at (MAX, -MAX), fold every vertex in order.
    void leaf_bounds(uint32_t ni) {
        bvhgpu_node& nd = nodes[ni];
        float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
        float hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        for (uint32_t p = nd.left_first; p < nd.left_first + nd.primitive_count; ++p) {
            const float* t = tris + 9ull * p;
            for (int k = 0; k < 3; ++k) {
                lo[k] = min_nan_ignoring(lo[k], t[k]);
                lo[k] = min_nan_ignoring(lo[k], t[3 + k]);
                lo[k] = min_nan_ignoring(lo[k], t[6 + k]);
                hi[k] = max_nan_ignoring(hi[k], t[k]);
                hi[k] = max_nan_ignoring(hi[k], t[3 + k]);
                hi[k] = max_nan_ignoring(hi[k], t[6 + k]);
            }
        }
        std::memcpy(nd.bounds_min, lo, sizeof(lo));
        std::memcpy(nd.bounds_max, hi, sizeof(hi));
    }

    // find_best_split_plane (bvh.rs:333-394).  Returns the axis (-1 = none) and writes the
    // split position and its SAH cost.
    int best_split(const bvhgpu_node& nd, float* pos, float* cost) {
        const uint32_t b = nd.left_first, e = nd.left_first + nd.primitive_count;
        float cmin[3] = {1e30f, 1e30f, 1e30f};
        float cmax[3] = {1e-30f, 1e-30f, 1e-30f};
        for (uint32_t p = b; p < e; ++p) {
            for (int k = 0; k < 3; ++k) {
                cmin[k] = min_nan_ignoring(cmin[k], cent[3ull * p + k]);
                cmax[k] = max_nan_ignoring(cmax[k], cent[3ull * p + k]);
            }
        }
        Box bins[3][8];
        uint32_t cnt[3][8];
        float scale[3];
        bool active[3];
        for (int k = 0; k < 3; ++k) {
            active[k] = !(cmin[k] == cmax[k]);
            scale[k] = 8.0f / (cmax[k] - cmin[k]);
            for (int i = 0; i < 8; ++i) {
                box_zero(bins[k][i]);
                cnt[k][i] = 0;
            }
        }
        for (uint32_t p = b; p < e; ++p) {
            const float* t = tris + 9ull * p;
            for (int k = 0; k < 3; ++k) {
                if (!active[k]) continue;
                uint64_t bi = std::min<uint64_t>(7, f32_to_usize((cent[3ull * p + k] - cmin[k]) * scale[k]));
                cnt[k][bi] += 1;
                box_grow(bins[k][bi], t);
                box_grow(bins[k][bi], t + 3);
                box_grow(bins[k][bi], t + 6);
            }
        }
        int best_axis = -1;
        float best_pos = 0.0f, best_cost = FLT_MAX;
        for (int k = 0; k < 3; ++k) {
            if (!active[k]) continue;
            float la[7], ra[7];
            uint32_t lc[7], rc[7];
            Box lb, rb;
            box_zero(lb);
            box_zero(rb);
            uint32_t ls = 0, rs = 0;
            for (int i = 0; i < 7; ++i) {
                ls += cnt[k][i];
                lc[i] = ls;
                // Aabb::grow_aabb (aabb.rs:41-46): bins start as the zero box, never MAX.
                if (bins[k][i].lo[0] != FLT_MAX) {
                    box_grow(lb, bins[k][i].lo);
                    box_grow(lb, bins[k][i].hi);
                }
                la[i] = box_area(lb);
                rs += cnt[k][7 - i];
                rc[6 - i] = rs;
                if (bins[k][7 - i].lo[0] != FLT_MAX) {
                    box_grow(rb, bins[k][7 - i].lo);
                    box_grow(rb, bins[k][7 - i].hi);
                }
                ra[6 - i] = box_area(rb);
            }
            float step = (cmax[k] - cmin[k]) / 8.0f;
            for (int i = 0; i < 7; ++i) {
                float c = ((float)lc[i]) * la[i] + ((float)rc[i]) * ra[i];
                if (c < best_cost) {
                    best_axis = k;
                    best_pos = cmin[k] + step * ((float)(i + 1));
                    best_cost = c;
                }
            }
        }
        *pos = best_pos;
        *cost = best_cost;
        return best_axis;
    }

    void swap_prims(uint32_t a, uint32_t b) {
        float tmp[9];
        std::memcpy(tmp, tris + 9ull * a, sizeof(tmp));
        std::memcpy(tris + 9ull * a, tris + 9ull * b, sizeof(tmp));
        std::memcpy(tris + 9ull * b, tmp, sizeof(tmp));
        for (int k = 0; k < 3; ++k) std::swap(cent[3ull * a + k], cent[3ull * b + k]);
        if (perm) std::swap(perm[a], perm[b]);
    }

    // subdivide (bvh.rs:396-467) as a work list.  Returns false where the reference panics.
    bool run() {
        std::vector<uint32_t> work;
        work.push_back(0);
        while (!work.empty()) {
            uint32_t ni = work.back();
            work.pop_back();
            float pos, cost;
            int axis = best_split(nodes[ni], &pos, &cost);
            const bvhgpu_node nd = nodes[ni];
            Box nb;
            std::memcpy(nb.lo, nd.bounds_min, sizeof(nb.lo));
            std::memcpy(nb.hi, nd.bounds_max, sizeof(nb.hi));
            float leaf_cost = ((float)nd.primitive_count) * box_area(nb);  // calculate_node_cost (bvh.rs:398-403)
            if (cost >= leaf_cost) continue;
            if (axis < 0) return false;
            uint32_t i = nd.left_first;
            uint32_t j = i + nd.primitive_count - 1;
            while (i <= j) {
                if (cent[3ull * i + axis] < pos) {
                    i += 1;
                } else {
                    swap_prims(i, j);
                    if (j == 0) return false;  // u32 underflow in the reference
                    j -= 1;
                }
            }
            uint32_t left_count = i - nd.left_first;
            if (left_count == 0 || left_count == nd.primitive_count) continue;
            uint32_t l = nodes_used++;
            uint32_t r = nodes_used++;
            nodes[l].left_first = nd.left_first;
            nodes[l].primitive_count = left_count;
            nodes[r].left_first = i;
            nodes[r].primitive_count = nd.primitive_count - left_count;
            nodes[ni].left_first = l;
            nodes[ni].primitive_count = 0;
            leaf_bounds(l);
            leaf_bounds(r);
            work.push_back(r);
            work.push_back(l);
        }
        return true;
    }
};

}  // namespace

int build_bvh_host(bvhgpu_triangle* mesh, uint32_t n, bvhgpu_node* nodes_out, uint32_t* nodes_used,
                   uint32_t* perm_out) {
    static_assert(sizeof(bvhgpu_node) == 32, "node layout");
    static_assert(sizeof(bvhgpu_triangle) == 36, "triangle layout");
    if (!mesh || !nodes_out || !nodes_used || n == 0 || n > 0x7FFFFFFFu) return BVHGPU_ERR_INVALID_ARG;
    std::memset(nodes_out, 0, sizeof(bvhgpu_node) * 2ull * n);
    Builder b;
    b.tris = reinterpret_cast<float*>(mesh);
    b.n = n;
    b.nodes = nodes_out;
    if (perm_out) {
        for (uint32_t i = 0; i < n; ++i) perm_out[i] = i;
        b.perm = perm_out;
    }
    b.compute_centroids();
    nodes_out[0].left_first = 0;
    nodes_out[0].primitive_count = n;
    b.leaf_bounds(0);
    if (!b.run()) return BVHGPU_ERR_BUILD;
    *nodes_used = b.nodes_used;
    return BVHGPU_OK;
}

}  // namespace bvhgpu
