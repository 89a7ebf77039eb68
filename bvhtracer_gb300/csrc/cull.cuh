// Conservative culling of triangle clusters inside a leaf, with results identical to testing
// every triangle.
//
// The reference tests every triangle of a leaf with its float Moeller-Trumbore test
// (triangle.rs:42-72); its BVHs are nearly flat, so leaves hold thousands of triangles.  A leaf is
// split into clusters of spatially close triangles, and a cluster is skipped for a ray only when
// no triangle of it can be accepted by that float test with a t below the ray's current closest t
// -- so the closest hit (and its ties, decided by triangle index) is unchanged.
//
// Why skipping is safe.  For float inputs o, d, v0, e1, e2 the test computes (each step rounded,
// no fused multiply-add) n = d x e2, det = e1.n, s = o - v0, u = (s.n)/det, q = s x e1,
// v = (d.q)/det, t = (e2.q)/det and accepts when |det| >= 1e-4, 0 <= u <= 1, 0 <= v, u + v <= 1
// and t > 1e-4.  With the unit roundoff u0 = 2^-24, standard bounds for rounded cross and dot
// products give, against the same quantities in exact arithmetic (det*, u*, v*, t*: the exact
// intersection of the ray's line with the plane of the triangle v0 + a e1 + b e2,
// P* = o + t* d = v0 + u* e1 + v* e2):
//   |det - det*| <= E_det = 30 u0 E1 E2 D,  |s.n - s*.n*| <= E_u = 36 u0 S D E2,
//   |d.q - d.q*| <= E_v = 36 u0 S D E1,     |e2.q - e2.q*| <= E_t = 36 u0 S E1 E2,
// where D = max|d_i|, E1 / E2 bound |e1_i| / |e2_i| over the cluster and S bounds |o_i - x_i| over
// the cluster's box.  An accepted triangle has |det| >= 1e-4, so with rho = E_det / 1e-4 < 1 its
// exact barycentrics are within Du = ((E_u + E_det) / 1e-4 + 2 u0) / (1 - rho) and Dv of the
// parameter triangle, hence P* lies within R = 2 (Du + Dv + u0) (|e1| + |e2|) of the triangle,
// and t* <= t + Dt with Dt = ((E_t + t E_det) / 1e-4 + 2 u0 t) / (1 - rho).  P* is on the ray's
// line: if the line, up to t_best + Dt(t_best), misses the cluster's box grown by R, no triangle
// of the cluster is accepted below t_best.
//
// The evaluation below never culls more than that argument allows: every error term carries a
// factor 4, 1 / 1e-4 is rounded up to 10102 (>= 1 / 9.9e-5), 1 / (1 - x) is replaced by its upper
// bound 1 + 2x (x < 1/2), the stored box is widened outward by a relative 4 u0 (it is computed
// from rounded vertices v0 + e1, v0 + e2), and the grown box gets an extra absolute slack of
// 8 u0 (|lo| + |hi| + |o| + R) per axis, which exceeds the rounding of the slab arithmetic
// (lo - g - o) * (1 / d) with the IEEE reciprocal (<= 5.1 u0 (|lo| + R) + 3.1 u0 |o|).  Clusters
// with non-finite or huge coordinates (sealed with q = +inf), rays with a non-finite or huge
// component or a reciprocal 1 / d_i that overflows, and clusters where rho is not small are never
// culled.  Both properties were audited on the CPU against the float test on adversarial rays
// (aimed at edges, vertices and grazing the plane): no culled cluster held an accepted hit below
// t_best, and the measured errors stayed below 5 % of the margins.
#pragma once

#include <cfloat>
#include <cmath>
#include <cstdint>

#ifdef __CUDACC__
#define BVHGPU_HD __host__ __device__ __forceinline__
#else
#define BVHGPU_HD inline
#endif

namespace bvhgpu {

// Triangles per cluster: one packed pair per lane of a warp.
constexpr uint32_t kClusterTris = 64;

// One cluster as stored for the cull: its box (widened outward), p = E1 * E2 and q = E1 + E2,
// where E1 / E2 are the largest |component| of the triangles' edges e1 = v1 - v0, e2 = v2 - v0.
// q = +inf marks a cluster that is never culled.
struct ClusterBox {
    float lo[3];
    float p;
    float hi[3];
    float q;
};
static_assert(sizeof(ClusterBox) == 32, "cluster box layout");

constexpr float kCullUnit = 5.9604645e-8f;  // u0 = 2^-24
constexpr float kCullSafety = 4.0f;
constexpr float kCullInvDet = 10102.0f;     // >= 1 / 9.9e-5 > 1 / 1e-4
constexpr float kCullHuge = 1e15f;

BVHGPU_HD float cull_fmax(float a, float b) { return a > b ? a : b; }
BVHGPU_HD float cull_fmin(float a, float b) { return a < b ? a : b; }
BVHGPU_HD float cull_abs(float a) { return a < 0.0f ? -a : a; }
BVHGPU_HD float cull_down(float t) { return t < 0.0f ? t * (1.0f + 4.0f * kCullUnit) : t * (1.0f - 4.0f * kCullUnit); }
BVHGPU_HD float cull_up(float t) { return t < 0.0f ? t * (1.0f - 4.0f * kCullUnit) : t * (1.0f + 4.0f * kCullUnit); }

// Finishes a cluster from the raw min / max of its vertices v0, v0 + e1, v0 + e2 (as computed in
// float) and the raw E1, E2.  `finite` is false when any input was non-finite.
BVHGPU_HD ClusterBox cluster_seal(const float lo[3], const float hi[3], float e1max, float e2max, bool finite) {
    ClusterBox c;
    bool ok = finite && e1max < kCullHuge && e2max < kCullHuge;
    for (int i = 0; i < 3; ++i) {
        ok = ok && cull_abs(lo[i]) < kCullHuge && cull_abs(hi[i]) < kCullHuge;
        c.lo[i] = cull_down(lo[i]);
        c.hi[i] = cull_up(hi[i]);
    }
    c.p = e1max * e2max * (1.0f + 4.0f * kCullUnit);
    c.q = ok ? (e1max + e2max) * (1.0f + 4.0f * kCullUnit) : INFINITY;
    if (!ok) {  // keep the box finite so the cull arithmetic never sees inf - inf
        for (int i = 0; i < 3; ++i) c.lo[i] = c.hi[i] = 0.0f;
        c.p = 0.0f;
    }
    return c;
}

// The per-ray part of the cull (origin, direction, IEEE reciprocal, D-scaled error factors).
struct CullRay {
    float o[3], d[3], rd[3];
    float a_det;  // F 30 u0 D
    float b_uv;   // F 36 u0 D
    bool ok;
};

// rx, ry, rz: the IEEE reciprocals 1 / dx, 1 / dy, 1 / dz (the traversal's own).
BVHGPU_HD CullRay cull_ray_rd(float ox, float oy, float oz, float dx, float dy, float dz, float rx, float ry,
                              float rz) {
    CullRay r;
    r.o[0] = ox; r.o[1] = oy; r.o[2] = oz;
    r.d[0] = dx; r.d[1] = dy; r.d[2] = dz;
    r.rd[0] = rx; r.rd[1] = ry; r.rd[2] = rz;
    bool ok = true;
    float D = 0.0f;
    for (int i = 0; i < 3; ++i) {
        // a zero component is handled exactly; any other must have a finite reciprocal
        ok = ok && cull_abs(r.o[i]) < kCullHuge && cull_abs(r.d[i]) < kCullHuge &&
             (r.d[i] == 0.0f || cull_abs(r.rd[i]) < FLT_MAX);
        D = cull_fmax(D, cull_abs(r.d[i]));
    }
    r.ok = ok;
    r.a_det = kCullSafety * 30.0f * kCullUnit * D;
    r.b_uv = kCullSafety * 36.0f * kCullUnit * D;
    return r;
}

BVHGPU_HD CullRay cull_ray(float ox, float oy, float oz, float dx, float dy, float dz) {
    return cull_ray_rd(ox, oy, oz, dx, dy, dz, 1.0f / dx, 1.0f / dy, 1.0f / dz);
}

// True when no triangle of cluster c can be accepted by the reference's test for the ray with a
// t below t_best (t_best >= FLT_MAX, or NaN: no bound).
BVHGPU_HD bool cluster_culled(const ClusterBox& c, const CullRay& r, float t_best) {
    const float u0 = kCullUnit, K = kCullInvDet;
    if (!r.ok || !(c.q < kCullHuge)) return false;
    float S = 0.0f;
    for (int i = 0; i < 3; ++i)
        S = cull_fmax(S, cull_fmax(cull_abs(r.o[i] - c.lo[i]), cull_abs(r.o[i] - c.hi[i])));
    const float e_det = r.a_det * c.p;
    const float rho = e_det * K;
    if (!(rho < 0.25f)) return false;
    const float inv = 1.0f + 2.0f * (rho + 8.0f * u0);  // >= 1 / (1 - rho - 8 u0)
    const float e_uv = r.b_uv * S * c.q;                 // E_u + E_v
    const float duv = ((e_uv + 2.0f * e_det) * K + 8.0f * u0) * inv;
    const float R = 4.0f * (duv + 2.0f * u0) * c.q * 1.0001f + 1e-30f;
    if (!(R < kCullHuge)) return false;
    float thi = INFINITY;
    if (t_best < FLT_MAX) {
        const float e_t = kCullSafety * 36.0f * u0 * S * c.p;
        thi = (t_best + ((e_t + t_best * e_det) * K + 4.0f * u0 * t_best) * inv) * (1.0f + 8.0f * u0) + 1e-30f;
    }
    float tlo = -INFINITY;
    for (int i = 0; i < 3; ++i) {
        const float g = R + 8.0f * u0 * (cull_abs(c.lo[i]) + cull_abs(c.hi[i]) + cull_abs(r.o[i]) + R) + 1e-30f;
        const float lo = c.lo[i] - g, hi = c.hi[i] + g;
        if (r.d[i] == 0.0f) {
            if (r.o[i] < lo || r.o[i] > hi) return true;  // the line stays outside this slab
            continue;
        }
        const float t1 = (lo - r.o[i]) * r.rd[i], t2 = (hi - r.o[i]) * r.rd[i];
        tlo = cull_fmax(tlo, cull_fmin(t1, t2));
        thi = cull_fmin(thi, cull_fmax(t1, t2));
    }
    return tlo > thi;
}

}  // namespace bvhgpu
