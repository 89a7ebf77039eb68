// CPU oracle for the ray-BVH hot path of lambdaxymox/bvhtracer.
//
// TEST INFRASTRUCTURE ONLY: a restatement of the reference's Rust code used to
// check the CUDA library and as the timed CPU baseline.  Nothing in the
// product library links, loads or calls this file.
//
// Every function cites the reference file:line it restates (paths relative to
// the reference repository root; "BT" = bvhtracer/).  Floating-point operation
// order follows the reference exactly; the file must be compiled with
// -ffp-contract=off so that no multiply-add is fused (Rust never fuses).
//
// Third-party arithmetic: Vector3 dot/cross/normalize, component min/max and
// Matrix4x4 * Vector4 live in the `cglinalg` crate, which is not vendored in the
// reference (BT/Cargo.toml:20-22 asks for 0.16.10, no lockfile).  They are
// restated here as their published definitions: dot = (x*x' + y*y') + z*z',
// cross = (y*z'-z*y', z*x'-x*z', x*y'-y*x'), normalize = v / |v| per component,
// |v| = sqrt(dot(v,v)), M*v = ((m0*v0 + m1*v1) + m2*v2) + m3*v3 per row
// (column-major m[col][row]).  The exact-t known answers of the reference's
// tests pin dot/cross/normalize (see tests/test_oracle_known_answers.py).

#include "bvh_oracle.h"

#include <cfloat>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>
#include <algorithm>

namespace {

struct V3 {
    float x, y, z;
};

inline V3 mk(float x, float y, float z) { return V3{x, y, z}; }
inline V3 add(V3 a, V3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 sub(V3 a, V3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 muls(V3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
inline V3 neg(V3 a) { return mk(-a.x, -a.y, -a.z); }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float magnitude(V3 a) { return std::sqrt(dot(a, a)); }
inline V3 normalize(V3 a) {
    float m = magnitude(a);
    return mk(a.x / m, a.y / m, a.z / m);
}
inline float comp(V3 a, int axis) { return axis == 0 ? a.x : (axis == 1 ? a.y : a.z); }

// Rust f32::min / f32::max: NaN-ignoring.  The sign of a zero result is
// unspecified in Rust; this restatement (and the CUDA refit / TLAS kernels) keep
// the first argument on equality.
inline float rmin(float a, float b) {
    if (a != a) return b;
    if (b != b) return a;
    return (b < a) ? b : a;
}
inline float rmax(float a, float b) {
    if (a != a) return b;
    if (b != b) return a;
    return (b > a) ? b : a;
}
inline V3 vmin(V3 a, V3 b) { return mk(rmin(a.x, b.x), rmin(a.y, b.y), rmin(a.z, b.z)); }
inline V3 vmax(V3 a, V3 b) { return mk(rmax(a.x, b.x), rmax(a.y, b.y), rmax(a.z, b.z)); }

// BT/src/geometry/aabb.rs:11-19; Default = zero box (derive(Default)).
struct Aabb {
    V3 bmin{0.f, 0.f, 0.f};
    V3 bmax{0.f, 0.f, 0.f};
};

// aabb.rs:29-34
inline Aabb aabb_new_empty() {
    Aabb a;
    a.bmin = mk(FLT_MAX, FLT_MAX, FLT_MAX);
    a.bmax = mk(-FLT_MAX, -FLT_MAX, -FLT_MAX);
    return a;
}
// aabb.rs:36-39
inline void aabb_grow(Aabb& a, V3 p) {
    a.bmin = vmin(a.bmin, p);
    a.bmax = vmax(a.bmax, p);
}
// aabb.rs:41-46
inline void aabb_grow_aabb(Aabb& a, const Aabb& b) {
    if (b.bmin.x != FLT_MAX) {
        aabb_grow(a, b.bmin);
        aabb_grow(a, b.bmax);
    }
}
// aabb.rs:48-57
inline float aabb_area(const Aabb& a) {
    V3 e = sub(a.bmax, a.bmin);
    return e.x * e.y + e.y * e.z + e.z * e.x;
}

// BT/src/query/ray.rs:9-35
struct Ray {
    V3 o, d, rd;
    float t;
};
inline Ray ray_new(V3 o, V3 d, float t) {
    Ray r;
    r.o = o;
    r.d = d;
    r.rd = mk(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    r.t = t;
    return r;
}

// aabb.rs:65-84
inline bool aabb_intersect(const Aabb& b, const Ray& r, float* out) {
    float tx1 = (b.bmin.x - r.o.x) * r.rd.x;
    float tx2 = (b.bmax.x - r.o.x) * r.rd.x;
    float tmin = rmin(tx1, tx2);
    float tmax = rmax(tx1, tx2);
    float ty1 = (b.bmin.y - r.o.y) * r.rd.y;
    float ty2 = (b.bmax.y - r.o.y) * r.rd.y;
    tmin = rmax(tmin, rmin(ty1, ty2));
    tmax = rmin(tmax, rmax(ty1, ty2));
    float tz1 = (b.bmin.z - r.o.z) * r.rd.z;
    float tz2 = (b.bmax.z - r.o.z) * r.rd.z;
    tmin = rmax(tmin, rmin(tz1, tz2));
    tmax = rmin(tmax, rmax(tz1, tz2));
    if ((tmax >= tmin) && (tmin < r.t) && (tmax > 0.0f)) {
        *out = tmin;
        return true;
    }
    return false;
}

// BT/src/geometry/triangle.rs:11-17
struct Tri {
    V3 v[3];
};
inline Tri load_tri(const orc_tri& t) {
    Tri r;
    r.v[0] = mk(t.v[0], t.v[1], t.v[2]);
    r.v[1] = mk(t.v[3], t.v[4], t.v[5]);
    r.v[2] = mk(t.v[6], t.v[7], t.v[8]);
    return r;
}

// triangle.rs:33-39: (v0 + v1 + v2) * (1/3), one/three computed in f32.
inline V3 tri_centroid(const Tri& t) {
    const float one = 1.0f;
    const float three = one + one + one;
    const float one_third = one / three;
    return muls(add(add(t.v[0], t.v[1]), t.v[2]), one_third);
}

// triangle.rs:42-72 (Moeller-Trumbore); returns (min(ray.t, t), u, v).
inline bool tri_intersect(const Tri& tri, const Ray& ray, float* ot, float* ou, float* ov) {
    V3 e1 = sub(tri.v[1], tri.v[0]);
    V3 e2 = sub(tri.v[2], tri.v[0]);
    V3 n = cross(ray.d, e2);
    float area = dot(e1, n);
    const float threshold = 0.0001f;
    if (std::fabs(area) < threshold) return false;
    float f = 1.0f / area;
    V3 s = sub(ray.o, tri.v[0]);
    float u = f * dot(s, n);
    if (u < 0.0f || u > 1.0f) return false;
    V3 q = cross(s, e1);
    float v = f * dot(ray.d, q);
    if (v < 0.0f || u + v > 1.0f) return false;
    float t = f * dot(e2, q);
    if (t > threshold) {
        *ot = rmin(ray.t, t);
        *ou = u;
        *ov = v;
        return true;
    }
    return false;
}

// BT/src/model/bvh.rs:129-134 (32-byte node; leaf iff primitive_count > 0).
struct Node {
    Aabb aabb;
    uint32_t count = 0;
    uint32_t left_first = 0;
};

struct Bvh {
    std::vector<Node> nodes;
    std::vector<uint32_t> node_indices;
    uint32_t root = 0;
    uint32_t nodes_used = 0;
};

struct BuildError {};

// bvh.rs:317-330
void update_node_bounds(Bvh& b, const std::vector<Tri>& mesh, uint32_t ni) {
    Aabb a;
    a.bmin = mk(FLT_MAX, FLT_MAX, FLT_MAX);
    a.bmax = mk(-FLT_MAX, -FLT_MAX, -FLT_MAX);
    const Node& node = b.nodes[ni];
    uint32_t base = b.node_indices[node.left_first];
    for (uint32_t k = 0; k < node.count; ++k) {
        const Tri& p = mesh[base + k];
        a.bmin = vmin(a.bmin, p.v[0]);
        a.bmin = vmin(a.bmin, p.v[1]);
        a.bmin = vmin(a.bmin, p.v[2]);
        a.bmax = vmax(a.bmax, p.v[0]);
        a.bmax = vmax(a.bmax, p.v[1]);
        a.bmax = vmax(a.bmax, p.v[2]);
    }
    b.nodes[ni].aabb = a;
}

// Rust `f as usize` (saturating; NaN -> 0).
inline uint64_t as_usize(float f) {
    if (!(f > 0.0f)) return 0;
    if (f >= 18446744073709551616.0f) return UINT64_MAX;
    return (uint64_t)f;
}

struct Split {
    int axis;
    float position;
    float cost;
};

// bvh.rs:333-394
Split find_best_split_plane(const Bvh& b, const std::vector<Tri>& mesh, const Node& node) {
    const int BIN_COUNT = 8;
    Split best{-1, 0.0f, FLT_MAX};
    uint32_t base = b.node_indices[node.left_first];
    for (int axis = 0; axis < 3; ++axis) {
        float bounds_min = 1e30f;
        float bounds_max = 1e-30f;
        for (uint32_t k = 0; k < node.count; ++k) {
            float c = comp(tri_centroid(mesh[base + k]), axis);
            bounds_min = rmin(bounds_min, c);
            bounds_max = rmax(bounds_max, c);
        }
        if (bounds_min == bounds_max) continue;

        Aabb bin_box[BIN_COUNT];
        uint32_t bin_count[BIN_COUNT] = {0, 0, 0, 0, 0, 0, 0, 0};
        float bin_scale = ((float)BIN_COUNT) / (bounds_max - bounds_min);
        for (uint32_t k = 0; k < node.count; ++k) {
            const Tri& p = mesh[base + k];
            uint64_t possible = as_usize((comp(tri_centroid(p), axis) - bounds_min) * bin_scale);
            uint64_t idx = std::min<uint64_t>(BIN_COUNT - 1, possible);
            bin_count[idx] += 1;
            aabb_grow(bin_box[idx], p.v[0]);
            aabb_grow(bin_box[idx], p.v[1]);
            aabb_grow(bin_box[idx], p.v[2]);
        }

        float left_area[BIN_COUNT - 1], right_area[BIN_COUNT - 1];
        uint32_t left_count[BIN_COUNT - 1], right_count[BIN_COUNT - 1];
        Aabb left_box, right_box;  // zero boxes (Aabb::default)
        uint32_t left_sum = 0, right_sum = 0;
        for (int i = 0; i < BIN_COUNT - 1; ++i) {
            left_sum += bin_count[i];
            left_count[i] = left_sum;
            aabb_grow_aabb(left_box, bin_box[i]);
            left_area[i] = aabb_area(left_box);

            right_sum += bin_count[BIN_COUNT - 1 - i];
            right_count[BIN_COUNT - 2 - i] = right_sum;
            aabb_grow_aabb(right_box, bin_box[BIN_COUNT - 1 - i]);
            right_area[BIN_COUNT - 2 - i] = aabb_area(right_box);
        }

        float scale = (bounds_max - bounds_min) / ((float)BIN_COUNT);
        for (int i = 0; i < BIN_COUNT - 1; ++i) {
            float plane_cost = ((float)left_count[i]) * left_area[i] + ((float)right_count[i]) * right_area[i];
            if (plane_cost < best.cost) {
                best.axis = axis;
                best.position = bounds_min + scale * ((float)(i + 1));
                best.cost = plane_cost;
            }
        }
    }
    return best;
}

// bvh.rs:396-467 (recursive, depth-first: left subtree allocated before right).
void subdivide(Bvh& b, std::vector<Tri>& mesh, uint32_t ni) {
    Split s = find_best_split_plane(b, mesh, b.nodes[ni]);
    const Node node = b.nodes[ni];
    float no_split_cost = ((float)node.count) * aabb_area(node.aabb);
    if (s.cost >= no_split_cost) return;
    if (s.axis < 0) throw BuildError();  // `best_axis as usize` would index out of range

    uint32_t i = node.left_first;
    uint32_t j = i + node.count - 1;
    while (i <= j) {
        if (comp(tri_centroid(mesh[i]), s.axis) < s.position) {
            i += 1;
        } else {
            std::swap(mesh[i], mesh[j]);
            if (j == 0) throw BuildError();  // u32 underflow: the reference panics
            j -= 1;
        }
    }
    uint32_t left_count = i - node.left_first;
    if (left_count == 0 || left_count == node.count) return;

    uint32_t left = b.nodes_used++;
    uint32_t right = b.nodes_used++;
    b.nodes[left].left_first = b.nodes[ni].left_first;
    b.nodes[left].count = left_count;
    b.nodes[right].left_first = i;
    b.nodes[right].count = b.nodes[ni].count - left_count;
    b.nodes[ni].left_first = left;
    b.nodes[ni].count = 0;

    update_node_bounds(b, mesh, left);
    update_node_bounds(b, mesh, right);
    subdivide(b, mesh, left);
    subdivide(b, mesh, right);
}

// bvh.rs:510-541
bool bvh_build(std::vector<Tri>& mesh, Bvh& b) {
    size_t n = mesh.size();
    if (n == 0) return false;  // nodes[0] of an empty array: the reference panics
    b.node_indices.resize(n);
    for (size_t i = 0; i < n; ++i) b.node_indices[i] = (uint32_t)i;
    b.nodes.assign(2 * n, Node());
    b.root = 0;
    b.nodes_used = 2;
    b.nodes[0].left_first = 0;
    b.nodes[0].count = (uint32_t)n;
    update_node_bounds(b, mesh, 0);
    try {
        subdivide(b, mesh, 0);
    } catch (const BuildError&) {
        return false;
    }
    return true;
}

struct Hit {
    float t, u, v;
    uint32_t prim;
};

// bvh.rs:242-305 (Bvh::intersect_subtree).  Leaf triangles are tested against the
// ray as passed in (bvh.rs:251); boxes against the shrinking closest ray (:269-270);
// ties in entry distance visit the right child first (:271-275).
template <class NodeAt, class TriAt>
bool bvh_intersect_impl(NodeAt node_at, TriAt tri_at, uint32_t root, const Ray& ray, Hit* out,
                        orc_counters* c) {
    Node cur = node_at(root);
    std::vector<Node> stack;
    stack.reserve(64);
    Ray closest = ray;
    bool have = false;
    Hit best{0, 0, 0, 0};
    for (;;) {
        if (cur.count > 0) {
            if (c) c->leaves++;
            uint32_t base = cur.left_first;  // node_indices is the identity (bvh.rs:526-528)
            for (uint32_t k = 0; k < cur.count; ++k) {
                uint32_t prim = base + k;
                float t, u, v;
                if (c) c->tris++;
                if (tri_intersect(tri_at(prim), ray, &t, &u, &v)) {
                    if (t < closest.t) {
                        closest.t = t;
                        best = Hit{t, u, v, prim};
                        have = true;
                    }
                }
            }
            if (stack.empty()) break;
            cur = stack.back();
            stack.pop_back();
        } else {
            if (c) c->interior++;
            Node l = node_at(cur.left_first);
            Node r = node_at(cur.left_first + 1);
            float dl = 0, dr = 0;
            bool hl = aabb_intersect(l.aabb, closest, &dl);
            bool hr = aabb_intersect(r.aabb, closest, &dr);
            float kl = hl ? dl : FLT_MAX;
            float kr = hr ? dr : FLT_MAX;
            Node near_n, far_n;
            bool near_h, far_h;
            if (kl < kr) {
                near_n = l; near_h = hl; far_n = r; far_h = hr;
            } else {
                near_n = r; near_h = hr; far_n = l; far_h = hl;
            }
            if (near_h) {
                cur = near_n;
                if (far_h) stack.push_back(far_n);
                continue;
            }
            if (stack.empty()) break;
            cur = stack.back();
            stack.pop_back();
        }
    }
    if (closest.t < FLT_MAX && have) {
        *out = best;
        return true;
    }
    return false;
}

inline Node load_node(const orc_node& n) {
    Node r;
    r.aabb.bmin = mk(n.bounds_min[0], n.bounds_min[1], n.bounds_min[2]);
    r.aabb.bmax = mk(n.bounds_max[0], n.bounds_max[1], n.bounds_max[2]);
    r.count = n.primitive_count;
    r.left_first = n.left_first;
    return r;
}
inline void store_node(const Node& n, orc_node* o) {
    o->bounds_min[0] = n.aabb.bmin.x; o->bounds_min[1] = n.aabb.bmin.y; o->bounds_min[2] = n.aabb.bmin.z;
    o->bounds_max[0] = n.aabb.bmax.x; o->bounds_max[1] = n.aabb.bmax.y; o->bounds_max[2] = n.aabb.bmax.z;
    o->primitive_count = n.count;
    o->left_first = n.left_first;
}

inline Ray load_ray(const orc_ray& r) {
    return ray_new(mk(r.origin[0], r.origin[1], r.origin[2]),
                   mk(r.direction[0], r.direction[1], r.direction[2]), r.t);
}

const orc_hit MISS = {FLT_MAX, 0.0f, 0.0f, 0xFFFFFFFFu, 0xFFFFFFFFu};

void blas_trace_range(const orc_node* nodes, const orc_tri* mesh, const orc_ray* rays, orc_hit* hits,
                      orc_counters* counters, uint32_t begin, uint32_t end) {
    auto node_at = [nodes](uint32_t i) { return load_node(nodes[i]); };
    auto tri_at = [mesh](uint32_t i) { return load_tri(mesh[i]); };
    for (uint32_t i = begin; i < end; ++i) {
        Ray r = load_ray(rays[i]);
        Hit h{0, 0, 0, 0};
        orc_counters* c = counters ? &counters[i] : nullptr;
        if (c) std::memset(c, 0, sizeof(*c));
        if (bvh_intersect_impl(node_at, tri_at, 0, r, &h, c)) {
            hits[i] = orc_hit{h.t, h.u, h.v, h.prim, 0u};
        } else {
            hits[i] = MISS;
        }
    }
}

// --- TLAS (BT/src/scene/tlas.rs) -------------------------------------------------

struct TlasNode {
    Aabb aabb;          // Default: Aabb::new_empty (tlas.rs:48-56)
    uint32_t left_right = 0;
    uint32_t blas = 0;
};
// tlas.rs:17-32: new(l, r) = l + (r << 16); left() reads the HIGH half, right() the low.
inline uint32_t lr_new(uint32_t l, uint32_t r) { return l + (r << 16); }
inline uint32_t lr_left(uint32_t d) { return (d & 0xFFFF0000u) >> 16; }
inline uint32_t lr_right(uint32_t d) { return d & 0x0000FFFFu; }

// tlas.rs:179-202
int find_best_match(const std::vector<TlasNode>& nodes, const std::vector<int32_t>& list, int n, int a) {
    float smallest = FLT_MAX;
    int best_b = -1;
    for (int b = 0; b < n; ++b) {
        if (b != a) {
            V3 bmax = vmax(nodes[list[a]].aabb.bmax, nodes[list[b]].aabb.bmax);
            V3 bmin = vmin(nodes[list[a]].aabb.bmin, nodes[list[b]].aabb.bmin);
            V3 e = sub(bmax, bmin);
            float sa = e.x * e.y + e.y * e.z + e.z * e.x;
            if (sa < smallest) {
                smallest = sa;
                best_b = b;
            }
        }
    }
    return best_b;
}

// tlas.rs:204-250 (Tlas::rebuild) after TlasBuilder::build_for (tlas.rs:273-279).
bool tlas_build(const std::vector<Aabb>& bounds, std::vector<TlasNode>& nodes, uint32_t* nodes_used_out) {
    size_t count = bounds.size();
    if (count == 0) return false;  // nodes[0] of an empty array
    if (2 * count > 65536) return false;  // 16-bit child indices would wrap
    TlasNode def;
    def.aabb = aabb_new_empty();
    nodes.assign(2 * count, def);
    size_t node_index_count = count;
    std::vector<int32_t> node_indices(count, 0);
    int32_t nodes_used = 1;
    for (size_t i = 0; i < count; ++i) {
        node_indices[i] = nodes_used;
        nodes[nodes_used].aabb = bounds[i];
        nodes[nodes_used].blas = (uint32_t)i;
        nodes[nodes_used].left_right = 0;
        nodes_used += 1;
    }
    int a = 0;
    int b = find_best_match(nodes, node_indices, (int)node_index_count, a);
    while (node_index_count > 1) {
        if (b < 0) return false;  // node_indices[-1]: the reference panics
        int c = find_best_match(nodes, node_indices, (int)node_index_count, b);
        if (a == c) {
            int32_t ia = node_indices[a];
            int32_t ib = node_indices[b];
            TlasNode na = nodes[ia];
            TlasNode nb = nodes[ib];
            TlasNode& nn = nodes[nodes_used];
            nn.left_right = lr_new((uint32_t)ia, (uint32_t)ib);
            nn.aabb.bmin = vmin(na.aabb.bmin, nb.aabb.bmin);
            nn.aabb.bmax = vmax(na.aabb.bmax, nb.aabb.bmax);
            node_indices[a] = nodes_used;
            nodes_used += 1;
            node_indices[b] = node_indices[node_index_count - 1];
            node_index_count -= 1;
            b = find_best_match(nodes, node_indices, (int)node_index_count, a);
        } else {
            if (c < 0) return false;
            a = b;
            b = c;
        }
    }
    nodes[0] = nodes[node_indices[a]];
    *nodes_used_out = (uint32_t)nodes_used;
    return true;
}

// BT/src/transform.rs:219-234 through cglinalg Matrix4x4 * Vector4 (column-major m[col*4+row]).
inline V3 xf_point(const float* m, V3 p) {
    return mk(((m[0] * p.x + m[4] * p.y) + m[8] * p.z) + m[12] * 1.0f,
              ((m[1] * p.x + m[5] * p.y) + m[9] * p.z) + m[13] * 1.0f,
              ((m[2] * p.x + m[6] * p.y) + m[10] * p.z) + m[14] * 1.0f);
}
inline V3 xf_vector(const float* m, V3 p) {
    return mk(((m[0] * p.x + m[4] * p.y) + m[8] * p.z) + m[12] * 0.0f,
              ((m[1] * p.x + m[5] * p.y) + m[9] * p.z) + m[13] * 0.0f,
              ((m[2] * p.x + m[6] * p.y) + m[10] * p.z) + m[14] * 0.0f);
}

struct SceneView {
    const orc_tlas_node* tlas;
    const uint32_t* blas_of;
    const float* inv;
    uint32_t nobj;
    const orc_node* nodes;
    const uint32_t* node_off;
    const orc_tri* tris;
    const uint32_t* tri_off;
};

// tlas.rs:123-177 + scene_object.rs:78-89
bool scene_intersect_one(const SceneView& s, const Ray& ray, orc_hit* out, orc_counters* c, int inst_zero) {
    auto tnode = [&s](uint32_t i) {
        TlasNode n;
        const orc_tlas_node& o = s.tlas[i];
        n.aabb.bmin = mk(o.bounds_min[0], o.bounds_min[1], o.bounds_min[2]);
        n.aabb.bmax = mk(o.bounds_max[0], o.bounds_max[1], o.bounds_max[2]);
        n.left_right = o.left_right;
        n.blas = o.blas;
        return n;
    };
    TlasNode cur = tnode(0);
    std::vector<TlasNode> stack;
    Ray closest = ray;
    bool have = false;
    orc_hit best = MISS;
    for (;;) {
        if (cur.left_right == 0) {
            uint32_t obj = cur.blas;
            if (c) c->blas_entries++;
            const float* inv = s.inv + 16 * obj;
            V3 o = xf_point(inv, closest.o);
            V3 d = xf_vector(inv, closest.d);
            Ray mray = ray_new(o, d, closest.t);
            uint32_t bl = s.blas_of[obj];
            const orc_node* nb = s.nodes + s.node_off[bl];
            const orc_tri* tb = s.tris + s.tri_off[bl];
            auto node_at = [nb](uint32_t i) { return load_node(nb[i]); };
            auto tri_at = [tb](uint32_t i) { return load_tri(tb[i]); };
            Hit h{0, 0, 0, 0};
            if (bvh_intersect_impl(node_at, tri_at, 0, mray, &h, c)) {
                // Intersection.ray.t is the BLAS's closest t, i.e. h.t (bvh.rs:253, :297-300).
                if (h.t < closest.t) {
                    closest.t = h.t;
                    best = orc_hit{h.t, h.u, h.v, h.prim, inst_zero ? 0u : obj};
                    have = true;
                }
            }
            if (stack.empty()) break;
            cur = stack.back();
            stack.pop_back();
        } else {
            if (c) c->tlas_interior++;
            TlasNode l = tnode(lr_left(cur.left_right));
            TlasNode r = tnode(lr_right(cur.left_right));
            float dl = 0, dr = 0;
            bool hl = aabb_intersect(l.aabb, closest, &dl);
            bool hr = aabb_intersect(r.aabb, closest, &dr);
            float kl = hl ? dl : FLT_MAX;
            float kr = hr ? dr : FLT_MAX;
            TlasNode near_n, far_n;
            bool near_h, far_h;
            if (kl < kr) {
                near_n = l; near_h = hl; far_n = r; far_h = hr;
            } else {
                near_n = r; near_h = hr; far_n = l; far_h = hl;
            }
            if (near_h) {
                cur = near_n;
                if (far_h) stack.push_back(far_n);
                continue;
            }
            if (stack.empty()) break;
            cur = stack.back();
            stack.pop_back();
        }
    }
    if (closest.t < FLT_MAX && have) {
        *out = best;
        return true;
    }
    *out = MISS;
    return false;
}

// Cosine-weighted diffuse bounce (not in the reference; defined identically in the CUDA
// library).  Only correctly rounded IEEE operations (+ - * / sqrt) are used, so the CPU
// and GPU produce the same bits.  Marsaglia (1972) uniform sphere point q, direction
// normalize(n + q) with n the face-forward geometric normal.
inline uint32_t hash32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}
inline float rng_uniform(uint32_t key, uint32_t k) {
    uint32_t h = hash32(key + k * 0x9E3779B9u);
    return (float)(h >> 8) * (1.0f / 16777216.0f);
}

// From the hit point p and the (unnormalised) geometric normal n onward: normalise, face-forward
// against d, Marsaglia sphere point, direction normalize(n + q).
bool finish_bounce(V3 p, V3 n, V3 d_in, uint32_t seed, uint32_t pixel, orc_ray* out) {
    float nl = std::sqrt(dot(n, n));
    if (!(nl > 0.0f) || !(nl <= FLT_MAX)) return false;
    n = mk(n.x / nl, n.y / nl, n.z / nl);
    if (dot(n, d_in) > 0.0f) n = neg(n);
    uint32_t key = hash32(seed ^ hash32(pixel));
    V3 q = n;
    bool found = false;
    for (uint32_t k = 0; k < 32u && !found; ++k) {
        float x1 = 2.0f * rng_uniform(key, 2u * k) - 1.0f;
        float x2 = 2.0f * rng_uniform(key, 2u * k + 1u) - 1.0f;
        float s = x1 * x1 + x2 * x2;
        if (s < 1.0f && s > 0.0f) {
            float r = std::sqrt(1.0f - s);
            q = mk((2.0f * x1) * r, (2.0f * x2) * r, 1.0f - 2.0f * s);
            found = true;
        }
    }
    V3 d = add(n, q);
    float dl = std::sqrt(dot(d, d));
    if (dl < 1e-6f) {
        d = n;
    } else {
        d = mk(d.x / dl, d.y / dl, d.z / dl);
    }
    out->origin[0] = p.x; out->origin[1] = p.y; out->origin[2] = p.z;
    out->direction[0] = d.x; out->direction[1] = d.y; out->direction[2] = d.z;
    out->t = FLT_MAX;
    out->pad = 0;
    return true;
}

bool bounce_one(const Ray& prim, float t, const Tri& tri, uint32_t seed, uint32_t pixel, orc_ray* out) {
    V3 p = add(prim.o, muls(prim.d, t));  // Ray::interpolate (ray.rs:37-39)
    V3 e1 = sub(tri.v[1], tri.v[0]);
    V3 e2 = sub(tri.v[2], tri.v[0]);
    return finish_bounce(p, cross(e1, e2), prim.d, seed, pixel, out);
}

// Instanced hit: the model-space geometric normal goes to world space with the inverse-transpose
// of the instance transform (row r of inv^T is column r of the column-major inverse).
bool bounce_instanced(const Ray& prim, float t, const Tri& tri, const float* inv, uint32_t seed, uint32_t pixel,
                      orc_ray* out) {
    V3 p = add(prim.o, muls(prim.d, t));
    V3 e1 = sub(tri.v[1], tri.v[0]);
    V3 e2 = sub(tri.v[2], tri.v[0]);
    V3 m = cross(e1, e2);
    V3 n = mk((inv[0] * m.x + inv[1] * m.y) + inv[2] * m.z, (inv[4] * m.x + inv[5] * m.y) + inv[6] * m.z,
              (inv[8] * m.x + inv[9] * m.y) + inv[10] * m.z);
    return finish_bounce(p, n, prim.d, seed, pixel, out);
}

template <class F>
void parallel_for(uint32_t n, int nthreads, F f) {
    if (nthreads <= 1 || n < 1024) {
        f(0u, n);
        return;
    }
    std::vector<std::thread> th;
    // Interleaved chunks keep threads balanced on uneven per-ray costs.
    const uint32_t chunk = 256;
    uint32_t nchunks = (n + chunk - 1) / chunk;
    for (int t = 0; t < nthreads; ++t) {
        th.emplace_back([=]() {
            for (uint32_t c = (uint32_t)t; c < nchunks; c += (uint32_t)nthreads) {
                uint32_t b = c * chunk;
                uint32_t e = std::min(n, b + chunk);
                f(b, e);
            }
        });
    }
    for (auto& x : th) x.join();
}

}  // namespace

extern "C" {

int orc_triangle_intersect(const orc_tri* tri, const orc_ray* ray, float* t, float* u, float* v) {
    Tri tr = load_tri(*tri);
    Ray r = load_ray(*ray);
    return tri_intersect(tr, r, t, u, v) ? 1 : 0;
}

int orc_aabb_intersect(const float bmin[3], const float bmax[3], const orc_ray* ray, float* tmin) {
    Aabb b;
    b.bmin = mk(bmin[0], bmin[1], bmin[2]);
    b.bmax = mk(bmax[0], bmax[1], bmax[2]);
    Ray r = load_ray(*ray);
    return aabb_intersect(b, r, tmin) ? 1 : 0;
}

void orc_normalize(const float in[3], float out[3]) {
    V3 n = normalize(mk(in[0], in[1], in[2]));
    out[0] = n.x; out[1] = n.y; out[2] = n.z;
}

void orc_triangle_centroid(const orc_tri* tri, float out[3]) {
    V3 c = tri_centroid(load_tri(*tri));
    out[0] = c.x; out[1] = c.y; out[2] = c.z;
}

int orc_bvh_build(orc_tri* mesh, uint32_t n, orc_node* nodes_out, uint32_t* nodes_used) {
    if (!mesh || !nodes_out || !nodes_used) return ORC_ERR_ARG;
    std::vector<Tri> m(n);
    for (uint32_t i = 0; i < n; ++i) m[i] = load_tri(mesh[i]);
    Bvh b;
    if (!bvh_build(m, b)) return ORC_ERR_PANIC;
    for (uint32_t i = 0; i < n; ++i) {
        for (int k = 0; k < 3; ++k) {
            mesh[i].v[3 * k + 0] = m[i].v[k].x;
            mesh[i].v[3 * k + 1] = m[i].v[k].y;
            mesh[i].v[3 * k + 2] = m[i].v[k].z;
        }
    }
    for (size_t i = 0; i < b.nodes.size(); ++i) store_node(b.nodes[i], &nodes_out[i]);
    *nodes_used = b.nodes_used;
    return ORC_OK;
}

int orc_bvh_intersect(const orc_node* nodes, uint32_t nodes_used, const orc_tri* mesh, uint32_t n,
                      const orc_ray* rays, uint32_t nrays, orc_hit* hits, orc_counters* counters) {
    (void)nodes_used;
    (void)n;
    if (!nodes || !mesh || (!rays && nrays) || (!hits && nrays)) return ORC_ERR_ARG;
    blas_trace_range(nodes, mesh, rays, hits, counters, 0, nrays);
    return ORC_OK;
}

int orc_bvh_intersect_mt(const orc_node* nodes, uint32_t nodes_used, const orc_tri* mesh, uint32_t n,
                         const orc_ray* rays, uint32_t nrays, orc_hit* hits, int nthreads) {
    (void)nodes_used;
    (void)n;
    if (!nodes || !mesh || (!rays && nrays) || (!hits && nrays)) return ORC_ERR_ARG;
    parallel_for(nrays, nthreads, [&](uint32_t b, uint32_t e) {
        blas_trace_range(nodes, mesh, rays, hits, nullptr, b, e);
    });
    return ORC_OK;
}

// The two smallest distances at which `ray` meets a triangle of the BVH (the parity rule's
// near-tie check: rays whose two nearest hits lie within a relative 1e-5 are reported apart).
// Every node whose box the ray enters before the current second-best distance is visited
// (Aabb::intersect against a ray whose t is that distance), leaf triangles are tested with
// Triangle::intersect, and the two smallest t are kept; FLT_MAX where there is none.
void two_nearest(const orc_node* nodes, const orc_tri* mesh, const Ray& ray, float* t1, float* t2) {
    float a = FLT_MAX, b = FLT_MAX;
    std::vector<uint32_t> stack;
    stack.push_back(0);
    while (!stack.empty()) {
        const Node n = load_node(nodes[stack.back()]);
        stack.pop_back();
        Ray cull = ray;
        cull.t = b;
        float tmin = 0;
        if (!aabb_intersect(n.aabb, cull, &tmin)) continue;
        if (n.count > 0) {
            for (uint32_t k = 0; k < n.count; ++k) {
                float t, u, v;
                if (!tri_intersect(load_tri(mesh[n.left_first + k]), ray, &t, &u, &v)) continue;
                if (t < a) {
                    b = a;
                    a = t;
                } else if (t < b) {
                    b = t;
                }
            }
        } else {
            stack.push_back(n.left_first);
            stack.push_back(n.left_first + 1);
        }
    }
    *t1 = a;
    *t2 = b;
}

int orc_two_nearest_mt(const orc_node* nodes, const orc_tri* mesh, const orc_ray* rays, uint32_t nrays, float* t1,
                       float* t2, int nthreads) {
    if (!nodes || !mesh || (nrays && (!rays || !t1 || !t2))) return ORC_ERR_ARG;
    parallel_for(nrays, nthreads, [&](uint32_t b, uint32_t e) {
        for (uint32_t i = b; i < e; ++i) two_nearest(nodes, mesh, load_ray(rays[i]), &t1[i], &t2[i]);
    });
    return ORC_OK;
}

// Triangle::intersect_mut (triangle.rs:75-108) on an Intersection: same test, and on a hit
// ray.t = min(ray.t, t), interaction.{t, u, v} overwritten (u, v also when t is larger).
inline bool tri_intersect_mut(const Tri& tri, Ray& ray, float* it, float* iu, float* iv) {
    float t, u, v;
    Ray probe = ray;
    probe.t = INFINITY;  // min(inf, t) == t: the raw t, to which intersect_mut applies its own min
    if (!tri_intersect(tri, probe, &t, &u, &v)) return false;
    ray.t = rmin(ray.t, t);
    *it = ray.t;
    *iu = u;
    *iv = v;
    return true;
}

// Every ray against a triangle list in index order: mode 0 Triangle::intersect with a strict `<`
// (first smallest t), mode 1 Triangle::intersect_mut on one Intersection per ray (prim = last
// triangle that reported a hit).
int orc_triangles_intersect(const orc_tri* mesh, uint32_t ntris, const orc_ray* rays, uint32_t nrays, int mode,
                            orc_hit* hits) {
    if ((ntris && !mesh) || (nrays && (!rays || !hits))) return ORC_ERR_ARG;
    for (uint32_t i = 0; i < nrays; ++i) {
        Ray r = load_ray(rays[i]);
        float ct = r.t, hu = 0, hv = 0;
        uint32_t hp = 0xFFFFFFFFu;
        for (uint32_t k = 0; k < ntris; ++k) {
            const Tri tri = load_tri(mesh[k]);
            if (mode == 0) {
                float t, u, v;
                if (tri_intersect(tri, r, &t, &u, &v) && t < ct) {
                    ct = t;
                    hu = u;
                    hv = v;
                    hp = k;
                }
            } else {
                float t, u, v;
                if (tri_intersect_mut(tri, r, &t, &u, &v)) {
                    ct = t;
                    hu = u;
                    hv = v;
                    hp = k;
                }
            }
        }
        const bool hit = hp != 0xFFFFFFFFu && (mode == 1 || ct < FLT_MAX);
        hits[i] = hit ? orc_hit{ct, hu, hv, hp, 0u} : MISS;
    }
    return ORC_OK;
}

// ---- rigid-body physics (BT/src/physics/) -------------------------------------------------------
// Same operation order as the reference; f32 throughout.  powf is the host math library's (the
// reference calls f32::powf, i.e. the platform's powf); drag 1 and can_sleep false never reach it.

static void rb_point_to_world(const float* m, const float* p, float* out) {  // Transform3::transform_point
    for (int r = 0; r < 3; ++r) out[r] = ((m[r] * p[0] + m[4 + r] * p[1]) + m[8 + r] * p[2]) + m[12 + r] * 1.0f;
}
static float rb_mag(const float* v) { return std::sqrt((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]); }

// RigidBody::apply_force_at_point (rigid_body.rs:434-440)
static void rb_force_at_point(orc_rigid_body& b, const float* f, const float* p) {
    const float cm[3] = {p[0] - b.position[0], p[1] - b.position[1], p[2] - b.position[2]};
    for (int k = 0; k < 3; ++k) b.force_accum[k] += f[k];
    const float t[3] = {cm[1] * f[2] - cm[2] * f[1], cm[2] * f[0] - cm[0] * f[2], cm[0] * f[1] - cm[1] * f[0]};
    for (int k = 0; k < 3; ++k) b.torque_accum[k] += t[k];
    b.is_awake = 1;
}

// RigidBody::calculate_derived_data (rigid_body.rs:132-146), Transform3::from_translation_rotation
// (transform.rs:190-217), _transform_inertia_tensor (rigid_body.rs:30-70)
static void rb_derived(orc_rigid_body& b) {
    float* q = b.orientation;
    const float m = std::sqrt(((q[0] * q[0] + q[1] * q[1]) + q[2] * q[2]) + q[3] * q[3]);
    for (int k = 0; k < 4; ++k) q[k] = q[k] / m;
    const float s = q[0], x = q[1], y = q[2], z = q[3], one = 1.0f, two = one + one, zero = 0.0f;
    float rot[4][4];  // [col][row]
    rot[0][0] = one - two * y * y - two * z * z;
    rot[0][1] = two * x * y + two * s * z;
    rot[0][2] = two * x * z - two * s * y;
    rot[0][3] = zero;
    rot[1][0] = two * x * y - two * s * z;
    rot[1][1] = one - two * x * x - two * z * z;
    rot[1][2] = two * y * z + two * s * x;
    rot[1][3] = zero;
    rot[2][0] = two * x * z + two * s * y;
    rot[2][1] = two * y * z - two * s * x;
    rot[2][2] = one - two * x * x - two * y * y;
    rot[2][3] = zero;
    rot[3][0] = b.position[0];
    rot[3][1] = b.position[1];
    rot[3][2] = b.position[2];
    rot[3][3] = one;
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) b.transform[4 * c + r] = rot[c][r];
    float iit[3][3];  // [col][row]
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) iit[c][r] = b.inverse_inertia[3 * c + r];
    const float m00 = rot[0][0] * iit[0][0] + rot[1][0] * iit[0][1] + rot[2][0] * iit[0][2];
    const float m10 = rot[0][0] * iit[1][0] + rot[1][0] * iit[1][1] + rot[2][0] * iit[1][2];
    const float m20 = rot[0][0] * iit[2][0] + rot[1][0] * iit[2][1] + rot[2][0] * iit[2][2];
    const float m01 = rot[0][1] * iit[0][0] + rot[1][1] * iit[0][1] + rot[2][1] * iit[0][2];
    const float m11 = rot[0][1] * iit[1][0] + rot[1][1] * iit[1][1] + rot[2][1] * iit[1][2];
    const float m21 = rot[0][1] * iit[2][0] + rot[1][1] * iit[2][1] + rot[2][1] * iit[2][2];
    const float m02 = rot[0][2] * iit[0][0] + rot[1][2] * iit[0][1] + rot[2][2] * iit[0][2];
    const float m12 = rot[0][2] * iit[1][0] + rot[1][2] * iit[1][1] + rot[2][2] * iit[1][2];
    const float m22 = rot[0][2] * iit[2][0] + rot[1][2] * iit[2][1] + rot[2][2] * iit[2][2];
    float w[3][3];
    w[0][0] = m00 * rot[0][0] + m10 * rot[1][0] + m20 * rot[2][0];
    w[1][0] = m00 * rot[0][1] + m10 * rot[1][1] + m20 * rot[2][1];
    w[2][0] = m00 * rot[0][2] + m10 * rot[1][2] + m20 * rot[2][2];
    w[0][1] = m01 * rot[0][0] + m11 * rot[1][0] + m21 * rot[2][0];
    w[1][1] = m01 * rot[0][1] + m11 * rot[1][1] + m21 * rot[2][1];
    w[2][1] = m01 * rot[0][2] + m11 * rot[1][2] + m21 * rot[2][2];
    w[0][2] = m02 * rot[0][0] + m12 * rot[1][0] + m22 * rot[2][0];
    w[1][2] = m02 * rot[0][1] + m12 * rot[1][1] + m22 * rot[2][1];
    w[2][2] = m02 * rot[0][2] + m12 * rot[1][2] + m22 * rot[2][2];
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) b.inverse_inertia_world[3 * c + r] = w[c][r];
}

int orc_world_start_frame(orc_rigid_body* bodies, uint32_t n) {  // world.rs:43-48
    for (uint32_t i = 0; i < n; ++i) {
        for (int k = 0; k < 3; ++k) bodies[i].force_accum[k] = bodies[i].torque_accum[k] = 0.0f;
        rb_derived(bodies[i]);
    }
    return ORC_OK;
}

// World::run_physics (world.rs:56-59): ForceRegistry::apply_forces in registry order
// (force_registry.rs:73-77, force_generator.rs:52-59, 133-154), then RigidBody::integrate
// (rigid_body.rs:149-213) of every body.
int orc_world_step(orc_rigid_body* bodies, uint32_t n, const orc_force_generator* gens, uint32_t ngens, float d) {
    for (uint32_t g = 0; g < ngens; ++g) {
        const orc_force_generator& G = gens[g];
        if (G.body >= n) return ORC_ERR_ARG;
        orc_rigid_body& b = bodies[G.body];
        if (G.kind == 0) {
            if (b.inverse_mass >= 0.0f) {
                const float mass = b.inverse_mass == 0.0f ? FLT_MAX : 1.0f / b.inverse_mass;
                for (int k = 0; k < 3; ++k) b.force_accum[k] += G.gravity[k] * mass;
                b.is_awake = 1;
            }
        } else {
            if (G.other >= n) return ORC_ERR_ARG;
            float lws[3], ows[3];
            rb_point_to_world(b.transform, G.spring_point, lws);
            rb_point_to_world(bodies[G.other].transform, G.other_point, ows);
            const float disp[3] = {lws[0] - ows[0], lws[1] - ows[1], lws[2] - ows[2]};
            const float len = rb_mag(disp);
            const float fm = G.spring_constant * std::fabs(len - G.rest_length);
            const float m = rb_mag(disp);
            const float f[3] = {(disp[0] / m) * (-fm), (disp[1] / m) * (-fm), (disp[2] / m) * (-fm)};
            rb_force_at_point(b, f, lws);
        }
    }
    for (uint32_t i = 0; i < n; ++i) {
        orc_rigid_body& b = bodies[i];
        if (!b.is_awake) continue;
        for (int k = 0; k < 3; ++k) b.last_frame_acceleration[k] = b.acceleration[k] + b.force_accum[k] * b.inverse_mass;
        const float* W = b.inverse_inertia_world;
        float aa[3];
        for (int r = 0; r < 3; ++r) aa[r] = (W[r] * b.torque_accum[0] + W[3 + r] * b.torque_accum[1]) + W[6 + r] * b.torque_accum[2];
        for (int k = 0; k < 3; ++k) {
            b.velocity[k] += b.last_frame_acceleration[k] * d;
            b.rotation[k] += aa[k] * d;
        }
        const float ld = std::pow(b.linear_drag, d), ad = std::pow(b.angular_drag, d);
        for (int k = 0; k < 3; ++k) {
            b.velocity[k] *= ld;
            b.rotation[k] *= ad;
        }
        for (int k = 0; k < 3; ++k) b.position[k] += b.velocity[k] * d;
        // q = from_pure(rotation * d) * orientation (Hamilton product); orientation += q * 1/2
        const float p1 = b.rotation[0] * d, p2 = b.rotation[1] * d, p3 = b.rotation[2] * d, p0 = 0.0f;
        float* o = b.orientation;
        const float s2 = o[0], x2 = o[1], y2 = o[2], z2 = o[3];
        const float qs = p0 * s2 - p1 * x2 - p2 * y2 - p3 * z2;
        const float qx = p0 * x2 + p1 * s2 + p2 * z2 - p3 * y2;
        const float qy = p0 * y2 - p1 * z2 + p2 * s2 + p3 * x2;
        const float qz = p0 * z2 + p1 * y2 - p2 * x2 + p3 * s2;
        const float half = 0.5f;
        o[0] += qs * half;
        o[1] += qx * half;
        o[2] += qy * half;
        o[3] += qz * half;
        rb_derived(b);
        for (int k = 0; k < 3; ++k) b.force_accum[k] = b.torque_accum[k] = 0.0f;
        if (b.can_sleep) {
            const float* v = b.velocity;
            const float* r = b.rotation;
            const float cur = ((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]) + ((r[0] * r[0] + r[1] * r[1]) + r[2] * r[2]);
            const float bias = std::pow(0.5f, d);
            b.motion = bias * b.motion + (1.0f - bias) * cur;
            const float thr = 0.3f, ten = 10.0f;
            if (b.motion < thr) {
                b.is_awake = 0;
                for (int k = 0; k < 3; ++k) b.velocity[k] = b.rotation[k] = 0.0f;
            } else if (b.motion > ten * thr) {
                b.motion = ten * thr;
            }
        }
    }
    return ORC_OK;
}

// 3x3 determinant of rows rr, columns cc of a column-major 4x4, by the first row.
static float rb_det3(const float* m, const int* rr, const int* cc) {
    auto e = [&](int r, int c) { return m[4 * c + r]; };
    return (e(rr[0], cc[0]) * (e(rr[1], cc[1]) * e(rr[2], cc[2]) - e(rr[1], cc[2]) * e(rr[2], cc[1])) -
            e(rr[0], cc[1]) * (e(rr[1], cc[0]) * e(rr[2], cc[2]) - e(rr[1], cc[2]) * e(rr[2], cc[0]))) +
           e(rr[0], cc[2]) * (e(rr[1], cc[0]) * e(rr[2], cc[1]) - e(rr[1], cc[1]) * e(rr[2], cc[0]));
}

// SceneObject::update_transform (scene_object.rs:52-58): body transform * initial transform; its
// inverse by cofactors (the reference's Matrix4x4::inverse is not pinned by any test).
int orc_object_transforms(const orc_rigid_body* bodies, const uint32_t* body_of, const float* init, uint32_t nobj,
                          float* xf, float* inv) {
    for (uint32_t i = 0; i < nobj; ++i) {
        if (body_of[i] == 0xFFFFFFFFu) continue;
        const float* A = bodies[body_of[i]].transform;
        const float* B = init + 16 * (size_t)i;
        float P[16];
        for (int c = 0; c < 4; ++c)
            for (int r = 0; r < 4; ++r)
                P[4 * c + r] = ((A[r] * B[4 * c] + A[4 + r] * B[4 * c + 1]) + A[8 + r] * B[4 * c + 2]) +
                               A[12 + r] * B[4 * c + 3];
        float cof[16];
        for (int r = 0; r < 4; ++r)
            for (int c = 0; c < 4; ++c) {
                int rr[3], cc[3];
                for (int k = 0, j = 0; k < 4; ++k)
                    if (k != r) rr[j++] = k;
                for (int k = 0, j = 0; k < 4; ++k)
                    if (k != c) cc[j++] = k;
                const float d3 = rb_det3(P, rr, cc);
                cof[4 * r + c] = ((r + c) & 1) ? -d3 : d3;
            }
        const float det = ((P[0] * cof[0] + P[1] * cof[4]) + P[2] * cof[8]) + P[3] * cof[12];
        for (int k = 0; k < 16; ++k) xf[16 * (size_t)i + k] = P[k];
        for (int r = 0; r < 4; ++r)
            for (int c = 0; c < 4; ++c) inv[16 * (size_t)i + 4 * c + r] = cof[4 * c + r] / det;
    }
    return ORC_OK;
}

// bvh.rs:469-493
int orc_bvh_refit(orc_node* nodes, uint32_t nodes_used, const orc_tri* mesh, uint32_t n) {
    if (!nodes || !mesh) return ORC_ERR_ARG;
    (void)n;
    for (uint32_t idx = nodes_used; idx-- > 0;) {
        if (idx == 1) continue;
        Node node = load_node(nodes[idx]);
        if (node.count > 0) {
            Aabb a;
            a.bmin = mk(FLT_MAX, FLT_MAX, FLT_MAX);
            a.bmax = mk(-FLT_MAX, -FLT_MAX, -FLT_MAX);
            for (uint32_t k = 0; k < node.count; ++k) {
                Tri p = load_tri(mesh[node.left_first + k]);
                a.bmin = vmin(a.bmin, p.v[0]);
                a.bmin = vmin(a.bmin, p.v[1]);
                a.bmin = vmin(a.bmin, p.v[2]);
                a.bmax = vmax(a.bmax, p.v[0]);
                a.bmax = vmax(a.bmax, p.v[1]);
                a.bmax = vmax(a.bmax, p.v[2]);
            }
            node.aabb = a;
        } else {
            Node l = load_node(nodes[node.left_first]);
            Node r = load_node(nodes[node.left_first + 1]);
            node.aabb.bmin = vmin(l.aabb.bmin, r.aabb.bmin);
            node.aabb.bmax = vmax(l.aabb.bmax, r.aabb.bmax);
        }
        store_node(node, &nodes[idx]);
    }
    return ORC_OK;
}

uint32_t orc_bvh_depth(const orc_node* nodes, uint32_t nodes_used) {
    if (!nodes || nodes_used == 0) return 0;
    std::vector<std::pair<uint32_t, uint32_t>> st;
    st.push_back({0u, 1u});
    uint32_t best = 0;
    while (!st.empty()) {
        auto [i, d] = st.back();
        st.pop_back();
        best = std::max(best, d);
        if (nodes[i].primitive_count == 0) {
            st.push_back({nodes[i].left_first, d + 1});
            st.push_back({nodes[i].left_first + 1, d + 1});
        }
    }
    return best;
}

// scene_object.rs:60-75
void orc_object_bounds(const float model_min[3], const float model_max[3], const float xf[16],
                       float out_min[3], float out_max[3]) {
    Aabb nb = aabb_new_empty();
    for (int i = 0; i < 8; ++i) {
        float x = (i & 1) ? model_max[0] : model_min[0];
        float y = (i & 2) ? model_max[1] : model_min[1];
        float z = (i & 4) ? model_max[2] : model_min[2];
        aabb_grow(nb, xf_point(xf, mk(x, y, z)));
    }
    out_min[0] = nb.bmin.x; out_min[1] = nb.bmin.y; out_min[2] = nb.bmin.z;
    out_max[0] = nb.bmax.x; out_max[1] = nb.bmax.y; out_max[2] = nb.bmax.z;
}

int orc_tlas_build(const float* obj_min, const float* obj_max, uint32_t count, orc_tlas_node* nodes_out,
                   uint32_t* nodes_used) {
    if (!obj_min || !obj_max || !nodes_out || !nodes_used) return ORC_ERR_ARG;
    std::vector<Aabb> bounds(count);
    for (uint32_t i = 0; i < count; ++i) {
        bounds[i].bmin = mk(obj_min[3 * i], obj_min[3 * i + 1], obj_min[3 * i + 2]);
        bounds[i].bmax = mk(obj_max[3 * i], obj_max[3 * i + 1], obj_max[3 * i + 2]);
    }
    std::vector<TlasNode> nodes;
    uint32_t used = 0;
    if (!tlas_build(bounds, nodes, &used)) return ORC_ERR_PANIC;
    for (size_t i = 0; i < nodes.size(); ++i) {
        orc_tlas_node& o = nodes_out[i];
        o.bounds_min[0] = nodes[i].aabb.bmin.x; o.bounds_min[1] = nodes[i].aabb.bmin.y; o.bounds_min[2] = nodes[i].aabb.bmin.z;
        o.bounds_max[0] = nodes[i].aabb.bmax.x; o.bounds_max[1] = nodes[i].aabb.bmax.y; o.bounds_max[2] = nodes[i].aabb.bmax.z;
        o.left_right = nodes[i].left_right;
        o.blas = nodes[i].blas;
    }
    *nodes_used = used;
    return ORC_OK;
}

int orc_scene_intersect(const orc_tlas_node* tlas, uint32_t tlas_nodes_used, const uint32_t* blas_of,
                        const float* inv, uint32_t nobj, const orc_node* nodes, const uint32_t* node_off,
                        const orc_tri* tris, const uint32_t* tri_off, const orc_ray* rays, uint32_t nrays,
                        orc_hit* hits, orc_counters* counters, int reference_instance_zero) {
    (void)tlas_nodes_used;
    if (!tlas || !blas_of || !inv || !nodes || !node_off || !tris || !tri_off) return ORC_ERR_ARG;
    SceneView s{tlas, blas_of, inv, nobj, nodes, node_off, tris, tri_off};
    for (uint32_t i = 0; i < nrays; ++i) {
        orc_counters* c = counters ? &counters[i] : nullptr;
        if (c) std::memset(c, 0, sizeof(*c));
        scene_intersect_one(s, load_ray(rays[i]), &hits[i], c, reference_instance_zero);
    }
    return ORC_OK;
}

int orc_scene_intersect_mt(const orc_tlas_node* tlas, uint32_t tlas_nodes_used, const uint32_t* blas_of,
                           const float* inv, uint32_t nobj, const orc_node* nodes, const uint32_t* node_off,
                           const orc_tri* tris, const uint32_t* tri_off, const orc_ray* rays, uint32_t nrays,
                           orc_hit* hits, int nthreads) {
    (void)tlas_nodes_used;
    if (!tlas || !blas_of || !inv || !nodes || !node_off || !tris || !tri_off) return ORC_ERR_ARG;
    SceneView s{tlas, blas_of, inv, nobj, nodes, node_off, tris, tri_off};
    parallel_for(nrays, nthreads, [&](uint32_t b, uint32_t e) {
        for (uint32_t i = b; i < e; ++i) scene_intersect_one(s, load_ray(rays[i]), &hits[i], nullptr, 0);
    });
    return ORC_OK;
}

// BT/src/camera/camera.rs:994-1010 (get_ray_eye / get_ray_world).
void orc_camera_ray(const float corners[9], const float view_inv[16], float u, float v, orc_ray* out) {
    V3 tl = mk(corners[0], corners[1], corners[2]);
    V3 tr = mk(corners[3], corners[4], corners[5]);
    V3 bl = mk(corners[6], corners[7], corners[8]);
    V3 origin = mk(0.0f, 0.0f, 0.0f);
    V3 pixel = add(add(add(origin, tl), muls(sub(tr, tl), u)), muls(sub(bl, tl), v));
    V3 dir = normalize(sub(pixel, origin));
    V3 ow = xf_point(view_inv, origin);
    V3 dw = xf_vector(view_inv, dir);
    out->origin[0] = ow.x; out->origin[1] = ow.y; out->origin[2] = ow.z;
    out->direction[0] = dw.x; out->direction[1] = dw.y; out->direction[2] = dw.z;
    out->t = FLT_MAX;
    out->pad = 0;
}

// Accumulator / shader kinds (same values as include/bvhgpu.h).
enum { ACC_INTERSECTION = 0, ACC_DEPTH = 1, ACC_UV = 2, ACC_NORMAL = 3, ACC_TEXTURE = 4 };
enum { SH_RADIANCE = 0, SH_INTERSECTION = 1, SH_DEPTH = 2 };

static inline uint8_t rust_f32_as_u8(float x) {
    if (!(x > 0.0f)) return 0;  // NaN and negatives saturate to 0
    if (x >= 255.0f) return 255;
    return (uint8_t)x;
}
static inline uint64_t rust_f32_as_usize(float x) {  // saturating, NaN -> 0
    if (!(x > 0.0f)) return 0;
    if (x >= 18446744073709551616.0f) return UINT64_MAX;
    return (uint64_t)x;
}
static inline int32_t rust_f32_as_i32(float x) {
    if (x != x) return 0;
    if (x >= 2147483648.0f) return INT32_MAX;
    if (x <= -2147483648.0f) return INT32_MIN;
    return (int32_t)x;
}

// The accumulators of renderer.rs:134-334 for one camera ray's closest hit (`hit`, record h), then
// the pixel shaders of renderer.rs:116-222 into o[4].  normals / tex_coords / texels are the
// looked-up model's (per-triangle corner normals, 9 floats; corner texture coordinates, 6 floats;
// RGB8 texture, row-major tex_w x tex_h); normal_xf is the object transform applied to the
// interpolated normal (Transform3::transform_vector).  Returns ORC_ERR_ARG for an unknown kind.
static int shade_pixel(int accumulator, const float* P, int shader, const float* S, bool hit, const Hit& h,
                       const float* normals, const float* normal_xf, const float* tex_coords, const uint8_t* texels,
                       uint32_t tex_w, uint32_t tex_h, uint8_t* o, float* radiance) {
    V3 rad = mk(0, 0, 0);
    switch (accumulator) {
        case ACC_INTERSECTION:
            rad = hit ? mk(P[0], P[1], P[2]) : mk(P[3], P[4], P[5]);
            break;
        case ACC_DEPTH: {
            float t = hit ? h.t : FLT_MAX;
            rad = mk(t, t, t);
            break;
        }
        case ACC_UV:
            rad = hit ? mk(h.u, h.v, 1.0f - (h.u + h.v)) : mk(0, 0, 0);
            break;
        case ACC_NORMAL: {
            if (hit) {
                const float* nn = normals + 9 * (size_t)h.prim;
                V3 n0 = mk(nn[0], nn[1], nn[2]), n1 = mk(nn[3], nn[4], nn[5]), n2 = mk(nn[6], nn[7], nn[8]);
                float w0 = 1.0f - h.u - h.v;
                V3 nm = add(add(muls(n0, w0), muls(n1, h.u)), muls(n2, h.v));
                V3 nw = xf_vector(normal_xf, nm);
                V3 nz = normalize(nw);
                rad = muls(add(nz, mk(1.0f, 1.0f, 1.0f)), 0.5f);
            }
            break;
        }
        case ACC_TEXTURE: {
            if (hit) {
                const float* tc = tex_coords + 6 * (size_t)h.prim;
                const float w0 = 1.0f - h.u - h.v;
                // tex_coords[0] * (1 - u - v) + tex_coords[1] * u + tex_coords[2] * v
                const float uvx = (tc[0] * w0 + tc[2] * h.u) + tc[4] * h.v;
                const float uvy = (tc[1] * w0 + tc[3] * h.u) + tc[5] * h.v;
                const uint64_t iu = rust_f32_as_usize(uvx * (float)tex_w) % tex_w;
                const uint64_t iv = rust_f32_as_usize(uvy * (float)tex_h) % tex_h;
                const uint8_t* px = texels + 3 * (iv * tex_w + iu);
                const float sc = 1.0f / 256.0f;  // rgb8_to_rgb32f
                rad = mk((float)px[0] * sc, (float)px[1] * sc, (float)px[2] * sc);
            }
            break;
        }
        default:
            return ORC_ERR_ARG;
    }
    if (radiance) {
        radiance[0] = rad.x; radiance[1] = rad.y; radiance[2] = rad.z;
    }
    switch (shader) {
        case SH_RADIANCE:
            o[0] = rust_f32_as_u8(255.0f * rad.x);
            o[1] = rust_f32_as_u8(255.0f * rad.y);
            o[2] = rust_f32_as_u8(255.0f * rad.z);
            o[3] = 255;
            break;
        case SH_INTERSECTION: {
            // shader params: hit rgba, miss rgba (0..255)
            bool nz = !(rad.x == 0.0f && rad.y == 0.0f && rad.z == 0.0f);
            const float* c = nz ? S : S + 4;
            o[0] = (uint8_t)c[0]; o[1] = (uint8_t)c[1]; o[2] = (uint8_t)c[2]; o[3] = (uint8_t)c[3];
            break;
        }
        case SH_DEPTH: {
            float scale = S[0], offset = S[1];
            float t = rad.x;
            if (t < FLT_MAX) {
                uint32_t col = 255u - (uint32_t)rust_f32_as_i32((t - offset) * scale);
                uint32_t c = col * 0x010101u;
                o[0] = (uint8_t)((c & 0x00FF0000u) >> 16);
                o[1] = (uint8_t)((c & 0x0000FF00u) >> 8);
                o[2] = (uint8_t)(c & 0x000000FFu);
            } else {
                o[0] = 0; o[1] = 0; o[2] = 0;
            }
            o[3] = 255;
            break;
        }
        default:
            return ORC_ERR_ARG;
    }
    return ORC_OK;
}

// renderer.rs:345-384 (PathTracer::evaluate) with the accumulators of renderer.rs:134-286
// and the shaders of renderer.rs:116-222.  The frame is w x h with 8x8 tiles; the
// reference's fixed 80x80 tile grid is the w = h = 640 case.
// TextureMaterialAccumulator (renderer.rs:289-334) reads per-corner texture coordinates (6 floats
// per triangle) and an RGB8 texture (row-major, tex_w x tex_h) through TextureMaterial::evaluate
// (materials/material.rs:44-52).  For the normal accumulator the object transform comes in
// acc_params (16 floats).
int orc_render_textured(const float corners[9], const float view_inv[16], int width, int height, int accumulator,
                        const float* acc_params, int shader, const float* shader_params, const orc_node* nodes,
                        uint32_t nodes_used, const orc_tri* tris, uint32_t ntris, const float* normals,
                        const float* tex_coords, const uint8_t* texels, uint32_t tex_w, uint32_t tex_h,
                        uint8_t* rgba, float* radiance) {
    (void)nodes_used;
    (void)ntris;
    if (width <= 0 || height <= 0 || !nodes || !tris || !rgba) return ORC_ERR_ARG;
    if (accumulator == ACC_NORMAL && !normals) return ORC_ERR_ARG;
    if (accumulator == ACC_TEXTURE && (!tex_coords || !texels || tex_w == 0 || tex_h == 0)) return ORC_ERR_ARG;
    auto node_at = [nodes](uint32_t i) { return load_node(nodes[i]); };
    auto tri_at = [tris](uint32_t i) { return load_tri(tris[i]); };
    const float* P = acc_params;
    const float* S = shader_params;
    if ((accumulator == ACC_INTERSECTION || accumulator == ACC_NORMAL) && !P) return ORC_ERR_ARG;
    if ((shader == SH_INTERSECTION || shader == SH_DEPTH) && !S) return ORC_ERR_ARG;
    for (int y = 0; y < height; ++y) {
        for (int x = 0; x < width; ++x) {
            orc_ray rr;
            orc_camera_ray(corners, view_inv, (float)x / (float)width, (float)y / (float)height, &rr);
            Ray r = load_ray(rr);
            Hit h{0, 0, 0, 0};
            bool hit = bvh_intersect_impl(node_at, tri_at, 0, r, &h, nullptr);
            size_t pix = (size_t)y * width + x;
            int rc = shade_pixel(accumulator, P, shader, S, hit, h, normals, P, tex_coords, texels, tex_w, tex_h,
                                 rgba + 4 * pix, radiance ? radiance + 3 * pix : nullptr);
            if (rc != ORC_OK) return rc;
        }
    }
    return ORC_OK;
}

// PathTracer::evaluate over a whole Scene (renderer.rs:345-384 -> Scene::intersect, scene.rs:32-34,
// tlas.rs:123-177, scene_object.rs:78-89), accumulators of renderer.rs:134-334.  The normal and
// texture accumulators look up `scene.get_unchecked(instance_index)` with the instance and primitive
// indices of the hit's InstancePrimitiveIndex (renderer.rs:258-263, 312-317):
//  lookup 0 (the reference): Bvh::intersect packs instance 0 (InstancePrimitiveIndex::from_primitive,
//    bvh.rs:296, intersection.rs:63-66), so every hit reads object 0's model and transform, with the
//    primitive index masked to its 20 bits (intersection.rs:57-60); an index outside object 0's mesh
//    panics in the reference (slice index out of bounds) -> ORC_ERR_PANIC;
//  lookup 1: the hit's own object and primitive.
// Per BLAS bl: nodes at node_off[bl], triangles (and their normals / texture coordinates, 9 / 6 floats
// each) at tri_off[bl] with tri_count[bl] of them, texture at texel_off[bl] (bytes) of tex_w[bl] x
// tex_h[bl].  xf: object transforms (16 floats, column-major); inv: their cached inverses.
int orc_render_scene(const float corners[9], const float view_inv[16], int width, int height, int accumulator,
                     const float* acc_params, int shader, const float* shader_params, const orc_tlas_node* tlas,
                     const uint32_t* blas_of, const float* xf, const float* inv, uint32_t nobj,
                     const orc_node* nodes, const uint32_t* node_off, const orc_tri* tris, const uint32_t* tri_off,
                     const uint32_t* tri_count, const float* normals, const float* tex_coords, const uint8_t* texels,
                     const uint64_t* texel_off, const uint32_t* tex_w, const uint32_t* tex_h, int lookup,
                     uint8_t* rgba, float* radiance) {
    if (width <= 0 || height <= 0 || !tlas || !blas_of || !xf || !inv || !nodes || !node_off || !tris ||
        !tri_off || !tri_count || !rgba || nobj == 0)
        return ORC_ERR_ARG;
    if (accumulator == ACC_NORMAL && !normals) return ORC_ERR_ARG;
    if (accumulator == ACC_TEXTURE && (!tex_coords || !texels || !texel_off || !tex_w || !tex_h)) return ORC_ERR_ARG;
    const float* P = acc_params;
    const float* S = shader_params;
    if (accumulator == ACC_INTERSECTION && !P) return ORC_ERR_ARG;
    if ((shader == SH_INTERSECTION || shader == SH_DEPTH) && !S) return ORC_ERR_ARG;
    SceneView sv{tlas, blas_of, inv, nobj, nodes, node_off, tris, tri_off};
    for (int y = 0; y < height; ++y) {
        for (int x = 0; x < width; ++x) {
            orc_ray rr;
            orc_camera_ray(corners, view_inv, (float)x / (float)width, (float)y / (float)height, &rr);
            orc_hit oh;
            const bool hit = scene_intersect_one(sv, load_ray(rr), &oh, nullptr, 0);
            Hit h{oh.t, oh.u, oh.v, oh.prim};
            const float* nrm = nullptr;
            const float* tc = nullptr;
            const uint8_t* tex = nullptr;
            uint32_t tw = 0, th = 0;
            const float* oxf = xf;
            if (hit && (accumulator == ACC_NORMAL || accumulator == ACC_TEXTURE)) {
                const uint32_t obj = lookup ? oh.inst : 0u;
                const uint32_t prim = lookup ? oh.prim : (oh.prim & 0x000FFFFFu);
                const uint32_t bl = blas_of[obj];
                if (prim >= tri_count[bl]) return ORC_ERR_PANIC;
                h.prim = prim;
                oxf = xf + 16 * (size_t)obj;
                if (normals) nrm = normals + 9 * (size_t)tri_off[bl];
                if (tex_coords) tc = tex_coords + 6 * (size_t)tri_off[bl];
                if (accumulator == ACC_TEXTURE) {
                    tex = texels + texel_off[bl];
                    tw = tex_w[bl];
                    th = tex_h[bl];
                    if (tw == 0 || th == 0) return ORC_ERR_ARG;
                }
            }
            size_t pix = (size_t)y * width + x;
            int rc = shade_pixel(accumulator, P, shader, S, hit, h, nrm, oxf, tc, tex, tw, th, rgba + 4 * pix,
                                 radiance ? radiance + 3 * pix : nullptr);
            if (rc != ORC_OK) return rc;
        }
    }
    return ORC_OK;
}

int orc_render(const float corners[9], const float view_inv[16], int width, int height, int accumulator,
               const float* acc_params, int shader, const float* shader_params, const orc_node* nodes,
               uint32_t nodes_used, const orc_tri* tris, uint32_t ntris, const float* normals, uint8_t* rgba,
               float* radiance) {
    if (accumulator == ACC_TEXTURE) return ORC_ERR_ARG;
    return orc_render_textured(corners, view_inv, width, height, accumulator, acc_params, shader, shader_params,
                               nodes, nodes_used, tris, ntris, normals, nullptr, nullptr, 0, 0, rgba, radiance);
}

int orc_bounce_ray(const orc_ray* primary, const orc_hit* hit, const orc_tri* tri, uint32_t seed, uint32_t pixel,
                   orc_ray* out) {
    if (hit->prim == 0xFFFFFFFFu) return 0;
    return bounce_one(load_ray(*primary), hit->t, load_tri(*tri), seed, pixel, out) ? 1 : 0;
}

int orc_scene_bounce_rays(const uint32_t* blas_of, const float* inv, const orc_tri* tris, const uint32_t* tri_off,
                          const orc_ray* primaries, const orc_hit* hits, uint32_t nrays, uint32_t seed, orc_ray* out,
                          uint8_t* valid) {
    for (uint32_t i = 0; i < nrays; ++i) {
        valid[i] = 0;
        if (hits[i].prim == 0xFFFFFFFFu) continue;
        const uint32_t obj = hits[i].inst;
        const orc_tri* tb = tris + tri_off[blas_of[obj]];
        valid[i] = bounce_instanced(load_ray(primaries[i]), hits[i].t, load_tri(tb[hits[i].prim]), inv + 16 * obj,
                                    seed, i, &out[i]) ? 1 : 0;
    }
    return ORC_OK;
}

int orc_bounce_rays(const orc_ray* primaries, const orc_hit* hits, uint32_t nrays, const orc_tri* tris,
                    uint32_t seed, orc_ray* out, uint8_t* valid) {
    for (uint32_t i = 0; i < nrays; ++i) {
        valid[i] = 0;
        if (hits[i].prim == 0xFFFFFFFFu) continue;
        valid[i] = bounce_one(load_ray(primaries[i]), hits[i].t, load_tri(tris[hits[i].prim]), seed, i, &out[i]) ? 1 : 0;
    }
    return ORC_OK;
}

}  // extern "C"
