// Device-side building blocks shared by the bvhgpu kernels.
//
// Parity rule: every floating-point step that decides a hit follows the reference's
// Rust operation order (BT/src/geometry/{aabb,triangle}.rs) with explicit
// round-to-nearest intrinsics, so no multiply-add is ever fused and every division /
// square root is the correctly rounded IEEE one.  The library is also compiled with
// -fmad=false -prec-div=true -prec-sqrt=true -ftz=false.
#pragma once

#include <cfloat>
#include <cstdint>

#include <cuda_runtime.h>

#include "cull.cuh"

namespace bvhgpu {

// Device error flags (OR-ed into the context's error word).
constexpr uint32_t kErrStack = 1u;
constexpr uint32_t kErrSteps = 2u;
constexpr uint32_t kErrLookup = 4u;  // a render's shading lookup fell outside the model's data
constexpr uint32_t kErrDeadline = 8u;  // a persistent launch stopped at the context's deadline

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// A persistent launch's time budget (bvhgpu_set_deadline), kept in the two words after the
// context's error word (0: none).  A warp stops taking and tracing rays once its launch has run
// longer, raises kErrDeadline and leaves: no wait, so an expired launch ends promptly, and the host
// reports the launch's outputs as incomplete.
struct Deadline {
    unsigned long long end;  // globaltimer value at which the warp stops; 0: no deadline
    __device__ __forceinline__ void start(const uint32_t* err) {
        const unsigned long long budget = *reinterpret_cast<const volatile unsigned long long*>(err + 2);
        const unsigned long long now = global_ns();
        end = budget == 0ull ? 0ull : budget > ~0ull - now ? ~0ull : now + budget;  // saturating
    }
    // Warp-uniform: lane 0's clock decides.
    __device__ __forceinline__ bool expired(uint32_t* err) const {
        if (end == 0ull) return false;
        const bool late = __shfl_sync(0xFFFFFFFFu, global_ns() > end ? 1 : 0, 0) != 0;
        if (late && (threadIdx.x & 31u) == 0u) atomicOr(err, kErrDeadline);
        return late;
    }
};

constexpr uint32_t kMiss = 0xFFFFFFFFu;
constexpr float kThreshold = 0.0001f;  // num_traits::cast(0.0001_f64) (triangle.rs:47)

// GPU node: two float4, {bmin.xyz, left_first bits}, {bmax.xyz, count bits}.  A branch's two
// children are adjacent (right = left + 1, bvh.rs:111-113), so one child pair is 64 bytes.
struct GBlas {
    const float4* nodes;  // 2 float4 per node
    const float4* tris;   // 3 float4 per triangle: {v0, 0}, {e1 = v1 - v0, 0}, {e2 = v2 - v0, 0}
    // Triangle pairs (2p, 2p+1) interleaved for packed f32x2 math: 20 floats per pair, component
    // c of {v0x v0y v0z e1x e1y e1z e2x e2y e2z} of triangle 2p + h at float 2c + h.
    const ulonglong2* pairs;
    // Hidden trees of the large leaves (null when none): one uint2 per triangle index (rounded up
    // to even), read at a leaf's first triangle, {first, count} of the hidden root ({0, 0}: no
    // hidden tree); then one uint2 per hidden pair p >= (ntris + 1) / 2: the triangle indices of
    // its two slots (0xFFFFFFFF: padding).  Hidden nodes follow the reference's nodes_used nodes in
    // `nodes` (a node whose children start at or beyond nodes_used is hidden): an interior one has
    // 2 to 4 children, consecutive from `first`, and count = kHiddenInterior | (children - 1) << 28 |
    // its cone; a leaf has count = kHiddenLeaf | pairs and first = its first pair in `pairs`, after
    // the (ntris + 1) / 2 pairs in triangle order.
    const uint2* hx;
    // Cone records of the hidden trees, 2 float4 each: {axis xyz, cos_phi}, {sin_phi, nmin, Q, B}
    // (cull.cuh) -- one per hidden root and per hidden node at even depth; an interior hidden
    // node's cone covers all its triangles.
    const float4* cones;
    uint32_t nodes_used;
    uint32_t ntris;
    uint32_t root_count;  // root node meta (node 0)
    uint32_t root_first;
};

constexpr uint32_t kHiddenLeaf = 0x80000000u;
constexpr uint32_t kHiddenInterior = 0x40000000u;
constexpr uint32_t kConeMask = 0x0FFFFFFFu;
constexpr uint32_t kWideShift = 28;  // hidden interior count: bits 28-29 = children - 1 (2..4 children)
constexpr uint32_t kAnyCone = 0xFFFFFFFFu;  // TravT::lcone: the margins hold in the whole hidden tree
// Below this root-cone margin a ray keeps the root cone's margins in the whole hidden tree (the
// finer cones would cost more to evaluate than they save).
constexpr float kConeSwitchDuv = 0.05f;

// Interior: a reference branch (count 0) or a hidden one (kHiddenInterior | cone).
__host__ __device__ __forceinline__ bool node_interior(uint32_t cnt) { return cnt == 0u || (cnt >> 30) == 1u; }
__host__ __device__ __forceinline__ uint32_t hidden_table_u2(uint32_t ntris) { return (ntris + 1u) & ~1u; }
// Reference leaves with at least this many triangles get a hidden tree, whose leaves hold at most
// kHiddenLeafTris triangles (two packed pairs).
constexpr uint32_t kHiddenMinLeaf = 16;
constexpr uint32_t kHiddenLeafTris = 4;
static_assert(kHiddenMinLeaf > kHiddenLeafTris, "a hidden root is an interior node");

__host__ __device__ __forceinline__ uint32_t pairs_in_order(uint32_t ntris) { return (ntris + 1u) / 2u; }

struct GHit {
    float t, u, v;
    uint32_t prim, inst;
};
static_assert(sizeof(GHit) == 20, "hit record layout");

__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }

// cglinalg Vector3::dot: (x*x' + y*y') + z*z'.
__device__ __forceinline__ float dot3(float ax, float ay, float az, float bx, float by, float bz) {
    return fadd(fadd(fmul(ax, bx), fmul(ay, by)), fmul(az, bz));
}

// Ray::new recomputes 1/d with an IEEE division (ray.rs:23-31).
__device__ __forceinline__ float3 recip3(float3 d) {
    return make_float3(__frcp_rn(d.x), __frcp_rn(d.y), __frcp_rn(d.z));
}

// Aabb::intersect (aabb.rs:65-84).  fminf/fmaxf ignore a NaN operand exactly like Rust's
// f32::min/max; the result only feeds comparisons, so the sign of a zero is irrelevant.
__device__ __forceinline__ bool slab(float4 lo, float4 hi, float3 o, float3 rd, float t, float& tmin_out) {
    float tx1 = fmul(fsub(lo.x, o.x), rd.x);
    float tx2 = fmul(fsub(hi.x, o.x), rd.x);
    float tmin = fminf(tx1, tx2);
    float tmax = fmaxf(tx1, tx2);
    float ty1 = fmul(fsub(lo.y, o.y), rd.y);
    float ty2 = fmul(fsub(hi.y, o.y), rd.y);
    tmin = fmaxf(tmin, fminf(ty1, ty2));
    tmax = fminf(tmax, fmaxf(ty1, ty2));
    float tz1 = fmul(fsub(lo.z, o.z), rd.z);
    float tz2 = fmul(fsub(hi.z, o.z), rd.z);
    tmin = fmaxf(tmin, fminf(tz1, tz2));
    tmax = fminf(tmax, fmaxf(tz1, tz2));
    tmin_out = tmin;
    return (tmax >= tmin) && (tmin < t) && (tmax > 0.0f);
}

// Triangle::intersect (triangle.rs:42-72), Moeller-Trumbore in the reference's order, but
// evaluated without early exits (same decision, less divergence).  Returns the raw t; the
// caller accepts it iff t < closest_t, which equals the reference's
// `min(ray.t, t) < closest_ray.t` test because closest_ray.t never exceeds ray.t.
// IEEE round-to-nearest 1/x for the triangle test's `S::one() / area` (triangle.rs:51, 83): the
// hardware estimate rcp.approx refined by one Newton-Raphson step in fused multiply-adds
// (Markstein's method: e = 1 - x*y, exact in an FMA; y' = y + e*y).  Checked on a GB300 against
// CUDA's IEEE reciprocal __frcp_rn for every float with 1e-4 <= |x| < 2^126, both signs
// (2,338,099,666 values): identical bit for bit, at about half the cost.  Huge, infinite and NaN
// arguments take __frcp_rn itself; for |x| < 1e-4 the value is never used, because the test
// rejects the triangle on |area| < 1e-4.
__device__ __forceinline__ float rcp_approx(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rcp_tri(float x) {
    if (!(fabsf(x) < 0x1p126f)) return __frcp_rn(x);
    const float y = rcp_approx(x);
    return __fmaf_rn(__fmaf_rn(-x, y, 1.0f), y, y);
}

__device__ __forceinline__ bool tri_test(float4 v0, float4 e1, float4 e2, float3 o, float3 d, float& t,
                                         float& u, float& v) {
    float nx = fsub(fmul(d.y, e2.z), fmul(d.z, e2.y));
    float ny = fsub(fmul(d.z, e2.x), fmul(d.x, e2.z));
    float nz = fsub(fmul(d.x, e2.y), fmul(d.y, e2.x));
    float area = dot3(e1.x, e1.y, e1.z, nx, ny, nz);
    float f = rcp_tri(area);
    float sx = fsub(o.x, v0.x);
    float sy = fsub(o.y, v0.y);
    float sz = fsub(o.z, v0.z);
    u = fmul(f, dot3(sx, sy, sz, nx, ny, nz));
    float qx = fsub(fmul(sy, e1.z), fmul(sz, e1.y));
    float qy = fsub(fmul(sz, e1.x), fmul(sx, e1.z));
    float qz = fsub(fmul(sx, e1.y), fmul(sy, e1.x));
    v = fmul(f, dot3(d.x, d.y, d.z, qx, qy, qz));
    t = fmul(f, dot3(e2.x, e2.y, e2.z, qx, qy, qz));
    bool ok = !(fabsf(area) < kThreshold);
    ok = ok && !(u < 0.0f || u > 1.0f);
    ok = ok && !(v < 0.0f || fadd(u, v) > 1.0f);
    ok = ok && (t > kThreshold);
    return ok;
}

__device__ __forceinline__ uint32_t ubits(float f) { return __float_as_uint(f); }

// f32::min / f32::max: a NaN operand is ignored, and on equality the first operand is kept
// (the host build and the oracle use the same rule; it decides the sign of a zero result).
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

// Order-preserving map of a float to 32 bits with both zeros at one rank: the high half of the
// 64-bit keys with which the min / max folds of the reference (update_node_bounds, the SAH bins)
// are reduced in parallel -- the low half is the position in the fold's order, so among equal
// values the first in that order wins, as the sequential f32::min / f32::max keeps it.
__device__ __forceinline__ uint32_t ordered(float f) {
    uint32_t b = __float_as_uint(f);
    if (f == 0.0f) return 0x80000000u;
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ unsigned long long key_min(float f, uint32_t pos) {
    return ((unsigned long long)ordered(f) << 32) | pos;
}
__device__ __forceinline__ unsigned long long key_max(float f, uint32_t pos) {
    return ((unsigned long long)ordered(f) << 32) | (0xFFFFFFFFu - pos);
}

// Closest-hit traversal of one BLAS (bvh.rs:242-305): DFS with the far child pushed, near
// child = strictly smaller entry distance (ties -> right child), popped nodes are not
// re-culled (the reference does not re-test a popped node's box), leaf triangles in
// primitive order with a strict `<` update.  The visit order is identical to the
// reference's, so equal-t ties resolve to the same primitive.  The stack holds the far
// child's (count, first), so a pop needs no memory load.  Triangles are stored as
// {v0, e1 = v1 - v0, e2 = v2 - v0}; each edge is the single IEEE subtraction of
// triangle.rs:44-45, so precomputing it changes no bit.
enum StepResult { kStepContinue = 0, kStepFinished = 1, kStepBigLeaf = 2 };

// Leaf policy of a traversal launch (results never depend on it): a ray walks a leaf's hidden tree
// when its barycentric margin there is below max_duv; other leaves with more than big_leaf
// triangles are tested by the whole warp, smaller ones by their own lane.
struct LeafPolicy {
    uint32_t big_leaf;
    float max_duv;
};
constexpr LeafPolicy kDefaultPolicy = {16u, 0.5f};

// One lane's ray (world or model space) and its running closest hit.
struct LaneRay {
    float3 o, d, rd;
    float ct;  // closest_ray.t
    float hu, hv;
    uint32_t hp;
    bool hit;
    uint32_t inst_cur = 0;  // instance whose BLAS is being traversed (two-level traversal)
    uint32_t inst = 0;      // instance of the closest hit
};

__device__ __forceinline__ void test_leaf_lane(const float4* __restrict__ tris, uint32_t first, uint32_t cnt,
                                               LaneRay& r) {
    const float4* T = tris + 3ull * first;
    for (uint32_t k = 0; k < cnt; ++k) {
        float4 a = __ldg(T + 3 * k);
        float4 e1 = __ldg(T + 3 * k + 1);
        float4 e2 = __ldg(T + 3 * k + 2);
        float t, u, v;
        if (tri_test(a, e1, e2, r.o, r.d, t, u, v) && t < r.ct) {
            r.ct = t;
            r.hu = u;
            r.hv = v;
            r.hp = first + k;
            r.hit = true;
            r.inst = r.inst_cur;
        }
    }
}

// ---- packed f32x2 arithmetic (Blackwell) ---------------------------------------------------
// add/sub/mul.rn.f32x2 operate on two IEEE binary32 values with round-to-nearest each, i.e.
// exactly two of the scalar __fadd_rn / __fsub_rn / __fmul_rn above; no multiply-add is fused.
typedef unsigned long long f2;

__device__ __forceinline__ f2 f2_add(f2 a, f2 b) {
    f2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 f2_sub(f2 a, f2 b) {
    f2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
// Packed product RN(a*b) computed as fma.rn(a, b, z) with z = (-0, -0): a*b + (-0) is exactly a*b for
// every input (signed zeros included), so the result equals __fmul_rn per element.  z is read at run
// time so the compiler cannot prove it is -0: ptxas contracts a packed mul.rn.f32x2 that feeds an
// add/sub into one fused multiply-add (even with --fmad=false), which would change the rounding.
static __device__ unsigned long long g_neg_zero2 = 0x8000000080000000ull;
__device__ __forceinline__ f2 f2_neg_zero() { return *reinterpret_cast<volatile unsigned long long*>(&g_neg_zero2); }
__device__ __forceinline__ f2 f2_mul(f2 a, f2 b, f2 z) {
    f2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(z));
    return d;
}
__device__ __forceinline__ f2 f2_fma(f2 a, f2 b, f2 c) {  // two fused multiply-adds, one rounding each
    f2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ f2 f2_pack(float lo, float hi) {
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void f2_unpack(f2 v, float& lo, float& hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}

// Moeller-Trumbore (triangle.rs:42-72) on the two triangles of a pair at once, every step in
// the reference's order.  ok[h] is the reference's accept decision for triangle h.
// Moeller-Trumbore (triangle.rs:42-72) on the two triangles of a pair at once, every step in
// the reference's order, split in three parts so that several rays can share a loaded pair and
// rays with the same origin can share the origin terms s = o - v0, q = s x e1 and e2 . q (the
// same operations, computed once).
struct PairData {
    f2 V0X, V0Y, V0Z, E1X, E1Y, E1Z, E2X, E2Y, E2Z;
};
struct OriginTerms {
    f2 SX, SY, SZ, QX, QY, QZ, TN;
};
struct PairHit {
    bool okA, okB;
    float tA, tB, uA, uB, vA, vB;
};

__device__ __forceinline__ PairData load_pair(const ulonglong2* __restrict__ P) {
    ulonglong2 q0 = __ldg(P), q1 = __ldg(P + 1), q2 = __ldg(P + 2), q3 = __ldg(P + 3), q4 = __ldg(P + 4);
    PairData d;
    d.V0X = q0.x; d.V0Y = q0.y; d.V0Z = q1.x; d.E1X = q1.y; d.E1Y = q2.x;
    d.E1Z = q2.y; d.E2X = q3.x; d.E2Y = q3.y; d.E2Z = q4.x;
    return d;
}

__device__ __forceinline__ OriginTerms origin_terms(const PairData& p, f2 OX, f2 OY, f2 OZ, f2 Z) {
    OriginTerms o;
    o.SX = f2_sub(OX, p.V0X);  // s = ray.origin - v0
    o.SY = f2_sub(OY, p.V0Y);
    o.SZ = f2_sub(OZ, p.V0Z);
    o.QX = f2_sub(f2_mul(o.SY, p.E1Z, Z), f2_mul(o.SZ, p.E1Y, Z));  // q = s x e1
    o.QY = f2_sub(f2_mul(o.SZ, p.E1X, Z), f2_mul(o.SX, p.E1Z, Z));
    o.QZ = f2_sub(f2_mul(o.SX, p.E1Y, Z), f2_mul(o.SY, p.E1X, Z));
    o.TN = f2_add(f2_add(f2_mul(p.E2X, o.QX, Z), f2_mul(p.E2Y, o.QY, Z)), f2_mul(p.E2Z, o.QZ, Z));  // e2 . q
    return o;
}

__device__ __forceinline__ PairHit ray_terms(const PairData& p, const OriginTerms& o, f2 DX, f2 DY, f2 DZ, f2 Z,
                                             bool okA_in, bool okB_in) {
    f2 NX = f2_sub(f2_mul(DY, p.E2Z, Z), f2_mul(DZ, p.E2Y, Z));  // n = d x e2
    f2 NY = f2_sub(f2_mul(DZ, p.E2X, Z), f2_mul(DX, p.E2Z, Z));
    f2 NZ = f2_sub(f2_mul(DX, p.E2Y, Z), f2_mul(DY, p.E2X, Z));
    f2 A = f2_add(f2_add(f2_mul(p.E1X, NX, Z), f2_mul(p.E1Y, NY, Z)), f2_mul(p.E1Z, NZ, Z));  // e1 . n
    float aA, aB;
    f2_unpack(A, aA, aB);
    f2 F;  // 1 / area for both triangles (rcp_tri, the Newton step packed)
    if (fabsf(aA) < 0x1p126f && fabsf(aB) < 0x1p126f) {
        const f2 Y = f2_pack(rcp_approx(aA), rcp_approx(aB));
        const f2 E = f2_fma(A ^ 0x8000000080000000ull, Y, 0x3F8000003F800000ull);  // 1 - a*y
        F = f2_fma(E, Y, Y);
    } else {
        F = f2_pack(rcp_tri(aA), rcp_tri(aB));
    }
    f2 U = f2_mul(F, f2_add(f2_add(f2_mul(o.SX, NX, Z), f2_mul(o.SY, NY, Z)), f2_mul(o.SZ, NZ, Z)), Z);
    f2 V = f2_mul(F, f2_add(f2_add(f2_mul(DX, o.QX, Z), f2_mul(DY, o.QY, Z)), f2_mul(DZ, o.QZ, Z)), Z);
    f2 T = f2_mul(F, o.TN, Z);
    f2 UV = f2_add(U, V);
    PairHit h;
    float uvA, uvB;
    f2_unpack(U, h.uA, h.uB);
    f2_unpack(V, h.vA, h.vB);
    f2_unpack(T, h.tA, h.tB);
    f2_unpack(UV, uvA, uvB);
    h.okA = okA_in && !(fabsf(aA) < kThreshold) && !(h.uA < 0.0f || h.uA > 1.0f) && !(h.vA < 0.0f || uvA > 1.0f) &&
            (h.tA > kThreshold);
    h.okB = okB_in && !(fabsf(aB) < kThreshold) && !(h.uB < 0.0f || h.uB > 1.0f) && !(h.vB < 0.0f || uvB > 1.0f) &&
            (h.tB > kThreshold);
    return h;
}

// ---- traversal stacks -------------------------------------------------------------------------
// An entry is a pending far child, (count, first) of its node.
//
// SplitStack: the newest RK entries live in registers as a shift register (every index is a
// compile-time constant, so nothing goes to local memory); older entries spill to this thread's
// column of a shared-memory array (entry k at col[k * blockDim.x]: consecutive lanes hit
// consecutive 8-byte words, no bank conflicts).  A kernel using it takes
// kSharedEntries * 8 * blockDim.x bytes of dynamic shared memory and calls bind() once.
template <int RK, int SK>
struct SplitStack {
    static_assert(RK >= 1, "at least one register entry");
    static constexpr int kCap = RK + SK;
    static constexpr int kSharedEntries = SK;
    uint2 reg[RK];
    uint2* col;
    int sp;

    __device__ __forceinline__ void bind(uint2* smem) { col = smem + threadIdx.x; }
    __device__ __forceinline__ void clear() { sp = 0; }
    __device__ __forceinline__ bool empty() const { return sp == 0; }
    __device__ __forceinline__ bool full() const { return sp >= kCap; }
    __device__ __forceinline__ void push(uint2 e) {
        if (SK > 0 && sp >= RK) col[(sp - RK) * blockDim.x] = reg[RK - 1];
#pragma unroll
        for (int k = RK - 1; k > 0; --k) reg[k] = reg[k - 1];
        reg[0] = e;
        ++sp;
    }
    __device__ __forceinline__ uint2 pop() {
        const uint2 e = reg[0];
#pragma unroll
        for (int k = 0; k < RK - 1; ++k) reg[k] = reg[k + 1];
        if (SK > 0 && sp > RK) reg[RK - 1] = col[(sp - RK - 1) * blockDim.x];
        --sp;
        return e;
    }
};

// LocalStack: a plain per-thread array (local memory, cached in L1), for the rare deep trees.
template <int N>
struct LocalStack {
    static constexpr int kCap = N;
    static constexpr int kSharedEntries = 0;
    uint2 s[N];
    int sp;

    __device__ __forceinline__ void bind(uint2*) {}
    __device__ __forceinline__ void clear() { sp = 0; }
    __device__ __forceinline__ bool empty() const { return sp == 0; }
    __device__ __forceinline__ bool full() const { return sp >= N; }
    __device__ __forceinline__ void push(uint2 e) { s[sp++] = e; }
    __device__ __forceinline__ uint2 pop() { return s[--sp]; }
};

// A hidden leaf (np packed pairs from `first`, in spatial order) against the lane's own ray.  A
// triangle is taken when its t is below the closest t, or equal to it with a lower triangle index
// while the held hit came from the same reference leaf (`held`): the reference's in-order leaf loop
// keeps the lowest index among equal t, and a hit from an earlier leaf keeps equal t out.
__device__ __forceinline__ bool test_hidden_leaf(const GBlas& b, uint32_t first, uint32_t np, LaneRay& r, bool& held) {
    const uint2* hidx = b.hx + hidden_table_u2(b.ntris) - pairs_in_order(b.ntris);
    const f2 OX = f2_pack(r.o.x, r.o.x), OY = f2_pack(r.o.y, r.o.y), OZ = f2_pack(r.o.z, r.o.z);
    const f2 DX = f2_pack(r.d.x, r.d.x), DY = f2_pack(r.d.y, r.d.y), DZ = f2_pack(r.d.z, r.d.z);
    const f2 Z = f2_neg_zero();
    bool better = false;
    for (uint32_t q = 0; q < np; ++q) {
        const uint32_t p = first + q;
        const uint2 idx = __ldg(hidx + p);
        const PairData pd = load_pair(b.pairs + 5ull * p);
        const PairHit h = ray_terms(pd, origin_terms(pd, OX, OY, OZ, Z), DX, DY, DZ, Z, idx.x != kMiss, idx.y != kMiss);
        if (h.okA && (h.tA < r.ct || (h.tA == r.ct && held && idx.x < r.hp))) {
            r.ct = h.tA;
            r.hu = h.uA;
            r.hv = h.vA;
            r.hp = idx.x;
            held = true;
            better = true;
        }
        if (h.okB && (h.tB < r.ct || (h.tB == r.ct && held && idx.y < r.hp))) {
            r.ct = h.tB;
            r.hu = h.uB;
            r.hv = h.vB;
            r.hp = idx.y;
            held = true;
            better = true;
        }
    }
    if (better) {
        r.hit = true;
        r.inst = r.inst_cur;
    }
    return better;
}

// box_live of a hidden node for a ray whose margins are on (the only rays that walk hidden trees),
// with the common case -- no zero direction component -- as straight-line code.
__device__ __forceinline__ bool hidden_box(float4 lo, float4 hi, float3 rd, const LeafCull& lc, float& t_enter) {
    if (lc.zero == 0u) {
        const float x1 = fmaf(lo.x, rd.x, lc.slo[0]), x2 = fmaf(hi.x, rd.x, lc.shi[0]);
        const float y1 = fmaf(lo.y, rd.y, lc.slo[1]), y2 = fmaf(hi.y, rd.y, lc.shi[1]);
        const float z1 = fmaf(lo.z, rd.z, lc.slo[2]), z2 = fmaf(hi.z, rd.z, lc.shi[2]);
        const float tlo = fmaxf(fmaxf(lc.tlo, fminf(x1, x2)), fmaxf(fminf(y1, y2), fminf(z1, z2)));
        const float thi = fminf(fminf(lc.thi, fmaxf(x1, x2)), fminf(fmaxf(y1, y2), fmaxf(z1, z2)));
        t_enter = tlo;
        return tlo <= thi;
    }
    const float l[3] = {lo.x, lo.y, lo.z}, h[3] = {hi.x, hi.y, hi.z}, d[3] = {rd.x, rd.y, rd.z};
    return box_live(l, h, d, lc, t_enter);
}

// Per-ray work counters of the counting traversal (TravT<..., true>): what the ray fetched.
struct TraceCounts {
    uint32_t ref_nodes;    // reference interior nodes (each loads its two children, 64 B)
    uint32_t hid_boxes;    // hidden child boxes tested (32 B each; 2 to 4 per hidden interior node)
    uint32_t entries;      // hidden trees entered (the leaf's table entry, 32 B)
    uint32_t hid_pairs;    // hidden pairs tested (80 B + 8 B slot indices)
    uint32_t lane_tris;    // triangles of small reference leaves tested by the lane (48 B)
    uint32_t coop_tris;    // triangles of big reference leaves tested by the warp (40 B a triangle)
    uint32_t cone_switches;  // margins recomputed for another cone (2 x 16 B cone record)
};

template <class STK, bool COUNT = false>
struct TravT {
    static constexpr bool kCount = COUNT;
    STK stk;
    uint32_t cnt, first, steps, max_steps;
    LeafCull lc;         // the ray's margins in the hidden tree being walked, valid below cone `lcone`
    uint32_t lcone;      // the cone lc was computed for
    uint32_t leaf_cone;  // the hidden tree's root cone (its margins hold everywhere in the tree)
    bool held;           // the closest hit came from the reference leaf of that hidden tree
    TraceCounts cn;

    __device__ __forceinline__ void init(const GBlas& b) {
        stk.clear();
        cnt = b.root_count;
        first = b.root_first;
        steps = 0;
        max_steps = 2u * (b.nodes_used + b.ntris) + 16u;  // hidden nodes: fewer than ntris
        held = false;
        if constexpr (COUNT) cn = TraceCounts{0u, 0u, 0u, 0u, 0u, 0u, 0u};
    }

    __device__ __forceinline__ bool pop() {
        if (stk.empty()) return true;
        const uint2 e = stk.pop();
        cnt = e.x;
        first = e.y;
        return false;
    }

    __device__ __forceinline__ bool push(uint2 e, uint32_t* err) {
        if (stk.full()) {
            atomicOr(err, kErrStack);
            return false;
        }
        stk.push(e);
        return true;
    }

    // A leaf node (!node_interior(cnt)).  A hidden leaf is tested by the lane.  A reference leaf with a hidden
    // tree continues at the tree's root when the ray's margins (computed here) are narrow enough to
    // cull; other reference leaves with more than `pol.big_leaf` triangles are not tested here: the
    // step returns kStepBigLeaf with (first, cnt) describing the leaf, and the caller tests it
    // (warp-cooperatively) and then calls pop().
    __device__ __forceinline__ StepResult leaf(const GBlas& b, LaneRay& r, LeafPolicy pol) {
        if (cnt & kHiddenLeaf) {
            if constexpr (COUNT) cn.hid_pairs += cnt & ~kHiddenLeaf;
            if (test_hidden_leaf(b, first, cnt & ~kHiddenLeaf, r, held)) lc.thi = leaf_thi(lc, r.ct);
            return pop() ? kStepFinished : kStepContinue;
        }
        if (b.hx != nullptr && pol.max_duv > 0.0f) {
            const uint2 e = __ldg(b.hx + first);
            if (e.x != 0u) {
                const uint32_t c = e.y & kConeMask;
                lc = cone_cull(b, r, c, pol);
                if (lc.on) {  // else: margins too wide for this ray, the leaf is tested in order
                    if constexpr (COUNT) ++cn.entries;
                    held = false;
                    leaf_cone = c;
                    lcone = lc.duv < kConeSwitchDuv ? kAnyCone : c;
                    first = e.x;  // the hidden root is always an interior node
                    cnt = e.y;
                    return kStepContinue;
                }
            }
        }
        if (cnt > pol.big_leaf) return kStepBigLeaf;
        if constexpr (COUNT) cn.lane_tris += cnt;
        test_leaf_lane(b.tris, first, cnt, r);
        return pop() ? kStepFinished : kStepContinue;
    }

    // A hidden interior node: its 2 to 4 children's boxes under the margins' exact cull (any
    // order is exact), the nearest entered, the other live ones pushed.
    __device__ __forceinline__ StepResult hidden_interior(const GBlas& b, LaneRay& r, LeafPolicy pol, uint32_t* err) {
        if (lcone != kAnyCone && (cnt & kConeMask) != lcone) {
            // a subtree under another cone: its own (tighter) margins, else the tree's root cone's
            lcone = cnt & kConeMask;
            lc = cone_cull(b, r, lcone, pol);
            if (!lc.on) lc = cone_cull(b, r, leaf_cone, pol);
            if constexpr (COUNT) ++cn.cone_switches;
        }
        const uint32_t k = ((cnt >> kWideShift) & 3u) + 1u;
        const float4* N = b.nodes + 2ull * first;
        if constexpr (COUNT) cn.hid_boxes += k;
        // the live children by entry distance (dead ones at +inf); three exchanges bring the nearest
        // first, which is entered, and the others are pushed (measured: the full 5-exchange sort
        // cost 0.6 % more on the icosphere frame than the order it buys)
        float t[4] = {INFINITY, INFINITY, INFINITY, INFINITY};
        uint2 e[4] = {make_uint2(0u, 0u), make_uint2(0u, 0u), make_uint2(0u, 0u), make_uint2(0u, 0u)};
        // children two at a time, both loads issued together (a child record past the last one is
        // always readable: the node array ends with a spare record)
#pragma unroll
        for (uint32_t c = 0; c < 4; c += 2) {
            if (c >= k) break;
            const float4 lo0 = __ldg(N + 2 * c), hi0 = __ldg(N + 2 * c + 1);
            const float4 lo1 = __ldg(N + 2 * c + 2), hi1 = __ldg(N + 2 * c + 3);
            float te;
            if (hidden_box(lo0, hi0, r.rd, lc, te)) {
                t[c] = te;
                e[c] = make_uint2(ubits(hi0.w), ubits(lo0.w));
            }
            if (c + 1 < k && hidden_box(lo1, hi1, r.rd, lc, te)) {
                t[c + 1] = te;
                e[c + 1] = make_uint2(ubits(hi1.w), ubits(lo1.w));
            }
        }
        auto cx = [&](int i, int j) {
            if (t[j] < t[i]) {
                const float tt = t[i];
                t[i] = t[j];
                t[j] = tt;
                const uint2 ee = e[i];
                e[i] = e[j];
                e[j] = ee;
            }
        };
        cx(0, 1);
        cx(2, 3);
        cx(0, 2);  // the nearest is now first; the pushed rest stays partly ordered (any order is exact)
        if (t[0] < INFINITY) {
#pragma unroll
            for (int i = 3; i >= 1; --i)
                if (t[i] < INFINITY && !push(e[i], err)) return kStepFinished;
            cnt = e[0].x;
            first = e[0].y;
            return kStepContinue;
        }
        return pop() ? kStepFinished : kStepContinue;
    }

    // An interior node (node_interior(cnt)): for a reference node its children's boxes under the
    // reference's slab test, the near child entered, the far one pushed (its visit order).
    __device__ __forceinline__ StepResult interior(const GBlas& b, LaneRay& r, LeafPolicy pol, uint32_t* err) {
        if (first >= b.nodes_used) return hidden_interior(b, r, pol, err);
        const float4* N = b.nodes + 2ull * first;
        float4 l0 = __ldg(N);
        float4 l1 = __ldg(N + 1);
        float4 r0 = __ldg(N + 2);
        float4 r1 = __ldg(N + 3);
        float dl, dr;
        bool hl, hr, left_near;
        if constexpr (COUNT) ++cn.ref_nodes;
        hl = slab(l0, l1, r.o, r.rd, r.ct, dl);
        hr = slab(r0, r1, r.o, r.rd, r.ct, dr);
        const float kl = hl ? dl : FLT_MAX;
        const float kr = hr ? dr : FLT_MAX;
        left_near = kl < kr;
        const bool near_hit = left_near ? hl : hr;
        const bool far_hit = left_near ? hr : hl;
        if (near_hit) {
            if (far_hit &&
                !push(left_near ? make_uint2(ubits(r1.w), ubits(r0.w)) : make_uint2(ubits(l1.w), ubits(l0.w)), err))
                return kStepFinished;
            cnt = left_near ? ubits(l1.w) : ubits(r1.w);
            first = left_near ? ubits(l0.w) : ubits(r0.w);
            return kStepContinue;
        }
        return pop() ? kStepFinished : kStepContinue;
    }

    __device__ __forceinline__ bool over_cap(uint32_t* err) {
        if (++steps > max_steps) {
            atomicOr(err, kErrSteps);
            return true;
        }
        return false;
    }

    // The ray's margins under cone record c (its Q, B, normal cone), thi from the closest t.
    __device__ __forceinline__ LeafCull cone_cull(const GBlas& b, const LaneRay& r, uint32_t c, LeafPolicy pol) const {
        const float4 a = __ldg(b.cones + 2ull * c), q = __ldg(b.cones + 2ull * c + 1);
        const LeafCone cone = {a.x, a.y, a.z, a.w, q.x, q.y};
        return leaf_cull(cull_ray_rd(r.o.x, r.o.y, r.o.z, r.d.x, r.d.y, r.d.z, r.rd.x, r.rd.y, r.rd.z), q.z, q.w, r.ct,
                         pol.max_duv, cone);
    }

    // Processes one node.
    __device__ __forceinline__ StepResult step(const GBlas& b, LaneRay& r, LeafPolicy pol, uint32_t* err) {
        if (over_cap(err)) return kStepFinished;
        return node_interior(cnt) ? interior(b, r, pol, err) : leaf(b, r, pol);
    }

    // Steps until the lane finishes or stops at a big leaf.  GROUPED: interior nodes in an inner
    // loop, then leaves, so that the lanes of a warp run the same kind of node together (faster for
    // warps of similar rays); otherwise one node of either kind per iteration (faster where a warp
    // mixes rays of different kinds, as the persistent kernels' warps do).
    template <bool GROUPED = false>
    __device__ __forceinline__ StepResult advance(const GBlas& b, LaneRay& r, LeafPolicy pol, uint32_t* err) {
        if (GROUPED) {
            for (;;) {
                while (node_interior(cnt)) {
                    if (over_cap(err)) return kStepFinished;
                    const StepResult s = interior(b, r, pol, err);
                    if (s != kStepContinue) return s;
                }
                if (over_cap(err)) return kStepFinished;
                const StepResult s = leaf(b, r, pol);
                if (s != kStepContinue) return s;
            }
        }
        for (;;) {
            const StepResult s = step(b, r, pol, err);
            if (s != kStepContinue) return s;
        }
    }
};

// Running best of one ray inside a cooperative leaf test (triangle index order kept: a pair's
// triangle A before B, strict `<`).  Only t and the triangle are kept; the winner's u, v are
// recomputed once after the warp reduction (reduce_and_take).
struct Best {
    float t;
    uint32_t k;
    __device__ __forceinline__ void take(const PairHit& h, uint32_t kA) {
        if (h.okA && h.tA < t) {
            t = h.tA;
            k = kA;
        }
        if (h.okB && h.tB < t) {
            t = h.tB;
            k = kA + 1u;
        }
    }
};

struct CoopRay {
    float ox, oy, oz, dx, dy, dz, ct;
};

__device__ __forceinline__ CoopRay bcast_ray(const LaneRay& r, int src) {
    const unsigned kAll = 0xFFFFFFFFu;
    CoopRay c;
    c.ox = __shfl_sync(kAll, r.o.x, src);
    c.oy = __shfl_sync(kAll, r.o.y, src);
    c.oz = __shfl_sync(kAll, r.o.z, src);
    c.dx = __shfl_sync(kAll, r.d.x, src);
    c.dy = __shfl_sync(kAll, r.d.y, src);
    c.dz = __shfl_sync(kAll, r.d.z, src);
    c.ct = __shfl_sync(kAll, r.ct, src);
    return c;
}

// Triangle k of the pair layout as {v0, e1, e2} (component c of triangle k at float 20 (k/2) + 2c + k%2).
__device__ __forceinline__ void load_pair_tri(const ulonglong2* __restrict__ pairs, uint32_t k, float4& v0, float4& e1,
                                              float4& e2) {
    const float* P = reinterpret_cast<const float*>(pairs) + 20ull * (k >> 1) + (k & 1u);
    v0 = make_float4(__ldg(P), __ldg(P + 2), __ldg(P + 4), 0.0f);
    e1 = make_float4(__ldg(P + 6), __ldg(P + 8), __ldg(P + 10), 0.0f);
    e2 = make_float4(__ldg(P + 12), __ldg(P + 14), __ldg(P + 16), 0.0f);
}

// Warp argmin of (t, k) -- minimum t, ties to the lowest triangle index -- then lane `src` takes
// the hit.  Its u, v are recomputed by the scalar test (tri_test: per element the same
// operations as the packed pair test, so t, u, v are the ones the loop saw).
__device__ __forceinline__ void reduce_and_take(Best b, const ulonglong2* __restrict__ pairs, int src, LaneRay& r) {
    const unsigned kAll = 0xFFFFFFFFu;
    const unsigned lane = threadIdx.x & 31u;
    float bt = b.t;
    uint32_t bk = b.k;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        float ot = __shfl_xor_sync(kAll, bt, off);
        uint32_t ok = __shfl_xor_sync(kAll, bk, off);
        if (ok != 0xFFFFFFFFu && (bk == 0xFFFFFFFFu || ot < bt || (ot == bt && ok < bk))) {
            bt = ot;
            bk = ok;
        }
    }
    if (bk != 0xFFFFFFFFu && (int)lane == src) {
        float4 v0, e1, e2;
        load_pair_tri(pairs, bk, v0, e1, e2);
        float t, u, v;
        tri_test(v0, e1, e2, r.o, r.d, t, u, v);
        r.ct = bt;
        r.hu = u;
        r.hv = v;
        r.hp = bk;
        r.hit = true;
        r.inst = r.inst_cur;
    }
}

// ---- warp-cooperative big-leaf test ------------------------------------------------------
// All 32 lanes test the ray(s) of lane(s) `src` against the leaf [first, first + cnt): lane k
// takes the triangle pairs pbeg + k, pbeg + k + 32, ... (coalesced 80-byte loads, two triangles
// per packed instruction), keeps its first strictly smallest t below the ray's closest t, and
// the warp reduces to the minimum t with ties going to the lowest triangle index -- exactly the
// triangle the reference's sequential loop (bvh.rs:250-258, strict `<` in index order) keeps.
// Must be called by all 32 lanes with the same arguments.
__device__ __forceinline__ void coop_leaf(const ulonglong2* __restrict__ pairs, uint32_t first, uint32_t cnt,
                                          int src, LaneRay& r) {
    const unsigned lane = threadIdx.x & 31u;
    const CoopRay c = bcast_ray(r, src);
    const f2 OX = f2_pack(c.ox, c.ox), OY = f2_pack(c.oy, c.oy), OZ = f2_pack(c.oz, c.oz);
    const f2 DX = f2_pack(c.dx, c.dx), DY = f2_pack(c.dy, c.dy), DZ = f2_pack(c.dz, c.dz);
    const f2 Z = f2_neg_zero();
    const uint32_t end = first + cnt;
    const uint32_t pbeg = first >> 1, pend = (end + 1) >> 1;
    Best b{c.ct, 0xFFFFFFFFu};
    for (uint32_t p = pbeg + lane; p < pend; p += 32u) {
        const uint32_t kA = 2u * p;
        PairData pd = load_pair(pairs + 5ull * p);
        OriginTerms ot = origin_terms(pd, OX, OY, OZ, Z);
        b.take(ray_terms(pd, ot, DX, DY, DZ, Z, kA >= first, kA + 1u < end), kA);
    }
    reduce_and_take(b, pairs, src, r);
}

// Two rays (lanes srcA, srcB) waiting on the same leaf: each loaded pair is tested against both,
// and when the rays share their origin bit for bit the origin terms are computed once.
__device__ __forceinline__ void coop_leaf2(const ulonglong2* __restrict__ pairs, uint32_t first, uint32_t cnt,
                                           int srcA, int srcB, LaneRay& r) {
    const unsigned lane = threadIdx.x & 31u;
    const CoopRay ca = bcast_ray(r, srcA);
    const CoopRay cb = bcast_ray(r, srcB);
    const bool same_o = __float_as_uint(ca.ox) == __float_as_uint(cb.ox) &&
                        __float_as_uint(ca.oy) == __float_as_uint(cb.oy) &&
                        __float_as_uint(ca.oz) == __float_as_uint(cb.oz);
    const f2 AOX = f2_pack(ca.ox, ca.ox), AOY = f2_pack(ca.oy, ca.oy), AOZ = f2_pack(ca.oz, ca.oz);
    const f2 ADX = f2_pack(ca.dx, ca.dx), ADY = f2_pack(ca.dy, ca.dy), ADZ = f2_pack(ca.dz, ca.dz);
    const f2 BOX = f2_pack(cb.ox, cb.ox), BOY = f2_pack(cb.oy, cb.oy), BOZ = f2_pack(cb.oz, cb.oz);
    const f2 BDX = f2_pack(cb.dx, cb.dx), BDY = f2_pack(cb.dy, cb.dy), BDZ = f2_pack(cb.dz, cb.dz);
    const f2 Z = f2_neg_zero();
    const uint32_t end = first + cnt;
    const uint32_t pbeg = first >> 1, pend = (end + 1) >> 1;
    Best ba{ca.ct, 0xFFFFFFFFu};
    Best bb{cb.ct, 0xFFFFFFFFu};
    if (same_o) {
        for (uint32_t p = pbeg + lane; p < pend; p += 32u) {
            const uint32_t kA = 2u * p;
            const bool va = kA >= first, vb = kA + 1u < end;
            PairData pd = load_pair(pairs + 5ull * p);
            OriginTerms ot = origin_terms(pd, AOX, AOY, AOZ, Z);
            ba.take(ray_terms(pd, ot, ADX, ADY, ADZ, Z, va, vb), kA);
            bb.take(ray_terms(pd, ot, BDX, BDY, BDZ, Z, va, vb), kA);
        }
    } else {
        for (uint32_t p = pbeg + lane; p < pend; p += 32u) {
            const uint32_t kA = 2u * p;
            const bool va = kA >= first, vb = kA + 1u < end;
            PairData pd = load_pair(pairs + 5ull * p);
            ba.take(ray_terms(pd, origin_terms(pd, AOX, AOY, AOZ, Z), ADX, ADY, ADZ, Z, va, vb), kA);
            bb.take(ray_terms(pd, origin_terms(pd, BOX, BOY, BOZ, Z), BDX, BDY, BDZ, Z, va, vb), kA);
        }
    }
    reduce_and_take(ba, pairs, srcA, r);
    reduce_and_take(bb, pairs, srcB, r);
}

// Four rays with the same origin (bit for bit) waiting on the same leaf: each loaded pair's origin
// terms once, tested against the four directions.
__device__ __forceinline__ void coop_leaf4(const ulonglong2* __restrict__ pairs, uint32_t first, uint32_t cnt,
                                           int s0, int s1, int s2, int s3, LaneRay& r) {
    const unsigned lane = threadIdx.x & 31u;
    const CoopRay c0 = bcast_ray(r, s0), c1 = bcast_ray(r, s1), c2 = bcast_ray(r, s2), c3 = bcast_ray(r, s3);
    const f2 OX = f2_pack(c0.ox, c0.ox), OY = f2_pack(c0.oy, c0.oy), OZ = f2_pack(c0.oz, c0.oz);
    const f2 Z = f2_neg_zero();
    const uint32_t end = first + cnt;
    const uint32_t pbeg = first >> 1, pend = (end + 1) >> 1;
    Best b0{c0.ct, 0xFFFFFFFFu}, b1{c1.ct, 0xFFFFFFFFu}, b2{c2.ct, 0xFFFFFFFFu}, b3{c3.ct, 0xFFFFFFFFu};
    for (uint32_t p = pbeg + lane; p < pend; p += 32u) {
        const uint32_t kA = 2u * p;
        const bool va = kA >= first, vb = kA + 1u < end;
        PairData pd = load_pair(pairs + 5ull * p);
        OriginTerms ot = origin_terms(pd, OX, OY, OZ, Z);
        b0.take(ray_terms(pd, ot, f2_pack(c0.dx, c0.dx), f2_pack(c0.dy, c0.dy), f2_pack(c0.dz, c0.dz), Z, va, vb), kA);
        b1.take(ray_terms(pd, ot, f2_pack(c1.dx, c1.dx), f2_pack(c1.dy, c1.dy), f2_pack(c1.dz, c1.dz), Z, va, vb), kA);
        b2.take(ray_terms(pd, ot, f2_pack(c2.dx, c2.dx), f2_pack(c2.dy, c2.dy), f2_pack(c2.dz, c2.dz), Z, va, vb), kA);
        b3.take(ray_terms(pd, ot, f2_pack(c3.dx, c3.dx), f2_pack(c3.dy, c3.dy), f2_pack(c3.dz, c3.dz), Z, va, vb), kA);
    }
    reduce_and_take(b0, pairs, s0, r);
    reduce_and_take(b1, pairs, s1, r);
    reduce_and_take(b2, pairs, s2, r);
    reduce_and_take(b3, pairs, s3, r);
}

__device__ __forceinline__ void load_ray(const float4* rays, uint32_t i, float3& o, float3& d, float& t) {
    float4 a = __ldg(rays + 2ull * i);
    float4 b = __ldg(rays + 2ull * i + 1);
    o = make_float3(a.x, a.y, a.z);
    t = a.w;
    d = make_float3(b.x, b.y, b.z);
}

__device__ __forceinline__ void store_hit(GHit* hits, uint32_t i, bool hit, float t, float u, float v,
                                          uint32_t prim, uint32_t inst) {
    GHit h;
    if (hit) {
        h.t = t; h.u = u; h.v = v; h.prim = prim; h.inst = inst;
    } else {
        h.t = FLT_MAX; h.u = 0.0f; h.v = 0.0f; h.prim = kMiss; h.inst = kMiss;
    }
    hits[i] = h;
}

// ---- bounce rays (not in the reference) ------------------------------------------------
// Same definition as the CPU oracle: lowbias32 hash, Marsaglia sphere point, direction
// normalize(n + q) around the face-forward geometric normal.  Only IEEE + - * / sqrt.
__device__ __forceinline__ uint32_t hash32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}
__device__ __forceinline__ float rng_uniform(uint32_t key, uint32_t k) {
    uint32_t h = hash32(key + k * 0x9E3779B9u);
    return fmul((float)(h >> 8), 1.0f / 16777216.0f);
}

// p = o + d*t (Ray::interpolate, ray.rs:37-39); triangle given as v0, e1, e2.
__device__ __forceinline__ bool bounce_dir(float3 o, float3 d, float t, float4 v0, float4 e1, float4 e2,
                                           uint32_t seed, uint32_t pixel, float3& po, float3& pd) {
    po = make_float3(fadd(o.x, fmul(d.x, t)), fadd(o.y, fmul(d.y, t)), fadd(o.z, fmul(d.z, t)));
    float nx = fsub(fmul(e1.y, e2.z), fmul(e1.z, e2.y));
    float ny = fsub(fmul(e1.z, e2.x), fmul(e1.x, e2.z));
    float nz = fsub(fmul(e1.x, e2.y), fmul(e1.y, e2.x));
    float nl = __fsqrt_rn(dot3(nx, ny, nz, nx, ny, nz));
    if (!(nl > 0.0f) || !(nl <= FLT_MAX)) return false;
    nx = __fdiv_rn(nx, nl);
    ny = __fdiv_rn(ny, nl);
    nz = __fdiv_rn(nz, nl);
    if (dot3(nx, ny, nz, d.x, d.y, d.z) > 0.0f) {
        nx = -nx; ny = -ny; nz = -nz;
    }
    uint32_t key = hash32(seed ^ hash32(pixel));
    float qx = nx, qy = ny, qz = nz;
    for (uint32_t k = 0; k < 32u; ++k) {
        float x1 = fsub(fmul(2.0f, rng_uniform(key, 2u * k)), 1.0f);
        float x2 = fsub(fmul(2.0f, rng_uniform(key, 2u * k + 1u)), 1.0f);
        float s = fadd(fmul(x1, x1), fmul(x2, x2));
        if (s < 1.0f && s > 0.0f) {
            float r = __fsqrt_rn(fsub(1.0f, s));
            qx = fmul(fmul(2.0f, x1), r);
            qy = fmul(fmul(2.0f, x2), r);
            qz = fsub(1.0f, fmul(2.0f, s));
            break;
        }
    }
    float dx = fadd(nx, qx), dy = fadd(ny, qy), dz = fadd(nz, qz);
    float dl = __fsqrt_rn(dot3(dx, dy, dz, dx, dy, dz));
    if (dl < 1e-6f) {
        pd = make_float3(nx, ny, nz);
    } else {
        pd = make_float3(__fdiv_rn(dx, dl), __fdiv_rn(dy, dl), __fdiv_rn(dz, dl));
    }
    return true;
}

// Bounce for an instanced hit: world hit point p = o + d t (o, d world space), geometric normal
// of the model-space triangle (e1 x e2) taken to world space with the inverse-transpose of the
// instance transform (row r of inv^T is column r of the column-major inverse), then the same
// face-forward + Marsaglia sampling as bounce_dir.  Identical on the CPU oracle.
__device__ __forceinline__ bool bounce_dir_instanced(float3 o, float3 d, float t, float4 e1, float4 e2,
                                                     const float* inv, uint32_t seed, uint32_t pixel, float3& po,
                                                     float3& pd) {
    po = make_float3(fadd(o.x, fmul(d.x, t)), fadd(o.y, fmul(d.y, t)), fadd(o.z, fmul(d.z, t)));
    const float mx = fsub(fmul(e1.y, e2.z), fmul(e1.z, e2.y));
    const float my = fsub(fmul(e1.z, e2.x), fmul(e1.x, e2.z));
    const float mz = fsub(fmul(e1.x, e2.y), fmul(e1.y, e2.x));
    float nx = fadd(fadd(fmul(inv[0], mx), fmul(inv[1], my)), fmul(inv[2], mz));
    float ny = fadd(fadd(fmul(inv[4], mx), fmul(inv[5], my)), fmul(inv[6], mz));
    float nz = fadd(fadd(fmul(inv[8], mx), fmul(inv[9], my)), fmul(inv[10], mz));
    float nl = __fsqrt_rn(dot3(nx, ny, nz, nx, ny, nz));
    if (!(nl > 0.0f) || !(nl <= FLT_MAX)) return false;
    nx = __fdiv_rn(nx, nl);
    ny = __fdiv_rn(ny, nl);
    nz = __fdiv_rn(nz, nl);
    if (dot3(nx, ny, nz, d.x, d.y, d.z) > 0.0f) {
        nx = -nx; ny = -ny; nz = -nz;
    }
    uint32_t key = hash32(seed ^ hash32(pixel));
    float qx = nx, qy = ny, qz = nz;
    for (uint32_t k = 0; k < 32u; ++k) {
        float x1 = fsub(fmul(2.0f, rng_uniform(key, 2u * k)), 1.0f);
        float x2 = fsub(fmul(2.0f, rng_uniform(key, 2u * k + 1u)), 1.0f);
        float s = fadd(fmul(x1, x1), fmul(x2, x2));
        if (s < 1.0f && s > 0.0f) {
            float r = __fsqrt_rn(fsub(1.0f, s));
            qx = fmul(fmul(2.0f, x1), r);
            qy = fmul(fmul(2.0f, x2), r);
            qz = fsub(1.0f, fmul(2.0f, s));
            break;
        }
    }
    float dx = fadd(nx, qx), dy = fadd(ny, qy), dz = fadd(nz, qz);
    float dl = __fsqrt_rn(dot3(dx, dy, dz, dx, dy, dz));
    if (dl < 1e-6f) {
        pd = make_float3(nx, ny, nz);
    } else {
        pd = make_float3(__fdiv_rn(dx, dl), __fdiv_rn(dy, dl), __fdiv_rn(dz, dl));
    }
    return true;
}

}  // namespace bvhgpu
