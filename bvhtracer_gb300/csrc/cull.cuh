// Conservative culling of groups of triangles inside a leaf, with results identical to testing
// every triangle.
//
// The reference tests every triangle of a leaf with its float Moeller-Trumbore test
// (triangle.rs:42-72); its BVHs are nearly flat, so leaves hold thousands of triangles.  The
// library puts a hidden tree of boxes over the triangles of each large leaf, and a box is skipped
// for a ray only when no triangle in it can be accepted by that float test with a t at or below the
// ray's current closest t -- so the closest hit (and its ties, decided by triangle index) is
// unchanged.
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
// where D = max|d_i|, E1 / E2 bound |e1_i| / |e2_i| and S bounds |o_i - x_i| over the triangles
// of the leaf.  An accepted triangle has |det| >= 1e-4, so with rho = E_det / 1e-4 < 1 its exact
// barycentrics are within Du = ((E_u + E_det) / 1e-4 + 2 u0) / (1 - rho) and Dv of the parameter
// triangle, hence every coordinate of P* is within R = 2 (Du + Dv + u0) (E1 + E2) of the
// triangle, and t* <= t + Dt with Dt = ((E_t + t E_det) / 1e-4 + 2 u0 t) / (1 - rho).  P* is on
// the ray's line: if the line, up to t_best + Dt(t_best), misses a box of triangles grown by R, no
// triangle in it is accepted at or below t_best.
//
// Both bounds are symmetric (|t - t*| <= Dt(t)), so an accepted hit (t > 1e-4) also has
// t* > 1e-4 - Dt(1e-4): parts of the line behind that need no test either.
//
// The same bounds hold with 1e-4 (1 - rho) replaced by any lower bound Dlo of |det*|.  A leaf also
// keeps a cone of its triangles' normal lines (an axis A with every |N_k . A| >= cos_phi |N_k| |A|,
// N_k = e1 x e2) and a lower bound nmin of |N_k|; det* = -d . N_k, so for a ray whose line makes an
// angle theta with A's, |det*| >= nmin |d| cos(theta + phi) when theta + phi < 90 degrees -- for
// triangles facing the ray this is far above 1e-4, and the margins shrink by the same factor.
//
// The leaf keeps Q >= E1 + E2 (so E1 E2 <= Q^2 / 4) and B >= every |coordinate| of its boxes (so
// S <= |o|_inf + B); the margins are computed once per ray and leaf (leaf_cull) and each box then
// costs one slab test (box_live).  The evaluation never culls more than the argument allows:
// every error term carries a factor 4, R another factor 2, every bound is rounded outward by a
// few u0 (the cone's cosines and lengths included), the stored boxes are widened outward by a relative 4 u0 (they are computed from the
// rounded vertices v0 + e1, v0 + e2), and the grown box gets an extra slack of
// 8 u0 (2 B + |o_i| + R) per axis, which exceeds the rounding of the slab arithmetic
// fma(lo, 1 / d, -(o + g) / d) with the IEEE reciprocal (<= 5.1 u0 R + 4.1 u0 |o| + 2.1 u0 |lo|).
// Leaves with a non-finite or huge coordinate (Q = +inf), rays with a non-finite or huge component
// or a tiny non-zero d_i (|1 / d_i| >= 1e20), and leaves without a positive Dlo are never culled.
// Both properties were audited on the CPU against the float test on adversarial rays (aimed at
// edges and vertices, grazing the plane, axis-aligned): no culled box held an accepted hit at or
// below t_best, and the measured errors stayed below 5 % of the margins.
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

constexpr float kCullUnit = 5.9604645e-8f;  // u0 = 2^-24
constexpr float kCullSafety = 4.0f;
constexpr float kCullHuge = 1e15f;

BVHGPU_HD float cull_fmax(float a, float b) { return a > b ? a : b; }
BVHGPU_HD float cull_fmin(float a, float b) { return a < b ? a : b; }
BVHGPU_HD float cull_abs(float a) { return a < 0.0f ? -a : a; }
BVHGPU_HD float cull_down(float t) { return t < 0.0f ? t * (1.0f + 4.0f * kCullUnit) : t * (1.0f - 4.0f * kCullUnit); }
BVHGPU_HD float cull_up(float t) { return t < 0.0f ? t * (1.0f - 4.0f * kCullUnit) : t * (1.0f + 4.0f * kCullUnit); }
#ifdef __CUDACC__
BVHGPU_HD float cull_fma(float a, float b, float c) { return fmaf(a, b, c); }
#else
BVHGPU_HD float cull_fma(float a, float b, float c) { return std::fma(a, b, c); }
#endif

// A group of triangles sealed for the cull: its box widened outward, and its contributions to the
// leaf's Q (E1 + E2, rounded up; +inf for a non-finite or huge group) and B (largest |coordinate|).
struct GroupSeal {
    float lo[3], hi[3];
    float q, b;
};

// From the raw min / max of a group's vertices v0, v0 + e1, v0 + e2 (as computed in float) and
// the raw largest |e1_i|, |e2_i|.  `finite` is false when any input was non-finite.
BVHGPU_HD GroupSeal group_seal(const float lo[3], const float hi[3], float e1max, float e2max, bool finite) {
    GroupSeal c;
    bool ok = finite && e1max < kCullHuge && e2max < kCullHuge;
    float b = 0.0f;
    for (int i = 0; i < 3; ++i) {
        ok = ok && cull_abs(lo[i]) < kCullHuge && cull_abs(hi[i]) < kCullHuge;
        c.lo[i] = cull_down(lo[i]);
        c.hi[i] = cull_up(hi[i]);
        b = cull_fmax(b, cull_fmax(cull_abs(c.lo[i]), cull_abs(c.hi[i])));
    }
    c.q = ok ? (e1max + e2max) * (1.0f + 4.0f * kCullUnit) : INFINITY;
    c.b = ok ? b : 0.0f;
    if (!ok)  // keep the box finite: the leaf is never culled anyway (q = inf)
        for (int i = 0; i < 3; ++i) c.lo[i] = c.hi[i] = 0.0f;
    return c;
}

// The per-ray part of the cull.
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
        // a zero component is handled exactly; any other needs |1 / d_i| < 1e20 (with |o|, B below
        // 1e15 no product of the slab arithmetic can overflow)
        ok = ok && cull_abs(r.o[i]) < kCullHuge && cull_abs(r.d[i]) < kCullHuge &&
             (r.d[i] == 0.0f || cull_abs(r.rd[i]) < 1e20f);
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

// The normal cone of a group of triangles (see above); nmin = 0 or cos_phi <= 0: none.  sin_phi is
// an upper bound of sqrt(1 - cos_phi^2) (cone_sin).
struct LeafCone {
    float ax, ay, az;
    float cos_phi, sin_phi, nmin;
};

BVHGPU_HD float cone_sin(float cos_phi) {
    return sqrtf(cull_fmax(0.0f, 1.0f - cos_phi * cos_phi * (1.0f - 4.0f * kCullUnit))) * (1.0f + 4.0f * kCullUnit);
}

// One triangle's contribution to a cone around axis (ax, ay, az): a lower bound of
// |N . A| / (|N| |A|) and of |N| for the exact N = e1 x e2, from the float edges.
BVHGPU_HD void cone_terms(const float e1[3], const float e2[3], float ax, float ay, float az, float& cos_lo,
                          float& n_lo) {
    const float u0 = kCullUnit;
    // N = e1 x e2 in float, each component within eN of the exact one
    const float n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
    const float en[3] = {3.0f * u0 * (cull_abs(e1[1] * e2[2]) + cull_abs(e1[2] * e2[1])),
                         3.0f * u0 * (cull_abs(e1[2] * e2[0]) + cull_abs(e1[0] * e2[2])),
                         3.0f * u0 * (cull_abs(e1[0] * e2[1]) + cull_abs(e1[1] * e2[0]))};
    const float a[3] = {ax, ay, az};
    float dot = 0.0f, dot_err = 0.0f, nn = 0.0f, n_err = 0.0f, aa = 0.0f;
    for (int i = 0; i < 3; ++i) {
        dot += n[i] * a[i];
        dot_err += (en[i] + 4.0f * u0 * cull_abs(n[i])) * cull_abs(a[i]);
        nn += n[i] * n[i];
        n_err += en[i];
        aa += a[i] * a[i];
    }
    const float nlen = sqrtf(nn), alen = sqrtf(aa);
    n_lo = (nlen * (1.0f - 8.0f * u0) - n_err) * (1.0f - 4.0f * u0);
    const float num = cull_abs(dot) - dot_err;
    const float den = (nlen * (1.0f + 8.0f * u0) + n_err) * alen * (1.0f + 8.0f * u0);
    cos_lo = (num > 0.0f && den > 0.0f && n_lo > 0.0f) ? num / den * (1.0f - 8.0f * u0) : -1.0f;
    if (!(n_lo > 0.0f)) n_lo = 0.0f;
}

// A lower bound of |d . N_k| for every triangle of a leaf with cone c (0 when it gives none).
BVHGPU_HD float cone_det_lo(const float d[3], const LeafCone& c) {
    const float u0 = kCullUnit;
    if (!(c.nmin > 0.0f) || !(c.cos_phi > 0.0f) || !(c.cos_phi <= 1.0f) || !(c.sin_phi >= 0.0f)) return 0.0f;
    const float a = d[0] * c.ax + d[1] * c.ay + d[2] * c.az;
    const float a_err = 4.0f * u0 * (cull_abs(d[0] * c.ax) + cull_abs(d[1] * c.ay) + cull_abs(d[2] * c.az));
    const float dd = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    const float AA = c.ax * c.ax + c.ay * c.ay + c.az * c.az;
    const float dlen = sqrtf(dd), alen = sqrtf(AA);
    const float cos_t = (cull_abs(a) - a_err) / (dlen * alen * (1.0f + 8.0f * u0)) * (1.0f - 4.0f * u0);
    if (!(cos_t > 0.0f)) return 0.0f;
    const float sin_t = sqrtf(cull_fmax(0.0f, 1.0f - cos_t * cos_t * (1.0f - 4.0f * u0))) * (1.0f + 4.0f * u0);
    const float sin_p = c.sin_phi;
    const float cs = (cos_t * c.cos_phi * (1.0f - 4.0f * u0) - sin_t * sin_p * (1.0f + 4.0f * u0)) * (1.0f - 4.0f * u0);
    if (!(cs > 0.0f)) return 0.0f;
    const float lo = c.nmin * dlen * (1.0f - 4.0f * u0) * cs * (1.0f - 64.0f * u0);
    return lo < FLT_MAX ? lo : 0.0f;
}

// The per-(ray, leaf) part: the grown slab planes folded with the origin, c_lo = o + g and
// c_hi = o - g per axis, pre-scaled by -1 / d where d is not zero (slab t = fma(x, 1/d, s)), the
// largest t that still matters (thi, from the ray's closest t) and the smallest (tlo: accepted hits
// have t > 1e-4, so t* > 1e-4 - Dt(1e-4)).  thi follows the closest t through leaf_thi.
// on = false: nothing of this leaf is culled for this ray.  zero: bit i set when d_i == 0.
struct LeafCull {
    float slo[3], shi[3];
    float thi, tlo;
    float dt0, dt1;  // Dt(t) <= dt0 + t dt1 (rounded up)
    float duv;       // the barycentric margin Du + Dv the planes were grown for
    bool on;
    uint32_t zero;
};

BVHGPU_HD float leaf_thi(const LeafCull& lc, float t_best) {
    if (!(t_best < FLT_MAX)) return INFINITY;
    return (t_best + (lc.dt0 + t_best * lc.dt1)) * (1.0f + 8.0f * kCullUnit) + 1e-30f;
}

// max_duv: the largest barycentric margin (Du + Dv) worth culling with; on = false above it.
BVHGPU_HD LeafCull leaf_cull(const CullRay& r, float Q, float B, float t_best, float max_duv, const LeafCone& cone) {
    const float u0 = kCullUnit;
    LeafCull lc;
    lc.on = false;
    lc.zero = 0u;
    for (int i = 0; i < 3; ++i) {
        if (r.d[i] == 0.0f) lc.zero |= 1u << i;
        lc.slo[i] = lc.shi[i] = 0.0f;
    }
    lc.thi = INFINITY;
    lc.tlo = -INFINITY;
    lc.dt0 = lc.dt1 = 0.0f;
    lc.duv = INFINITY;
    if (!r.ok || !(Q < kCullHuge) || !(B < kCullHuge)) return lc;
    const float oinf = cull_fmax(cull_abs(r.o[0]), cull_fmax(cull_abs(r.o[1]), cull_abs(r.o[2])));
    const float S = (oinf + B) * (1.0f + 4.0f * u0);
    const float P = 0.25f * Q * Q * (1.0f + 4.0f * u0);  // >= E1 E2
    const float e_det = r.a_det * P;
    // |det*| >= Dlo: accepted |det| >= 1e-4 (the float 0.0001f, triangle.rs:47), or the cone's bound
    const float d_acc = 0.0001f * (1.0f - 4.0f * u0) - e_det;
    const float d_cone = cone_det_lo(r.d, cone);
    const float Dlo = cull_fmax(d_acc, d_cone);
    if (!(Dlo > 0.0f)) return lc;
    const float KD = 1.0f / Dlo * (1.0f + 4.0f * u0);  // >= 1 / Dlo
    if (!(KD < kCullHuge)) return lc;
    const float e_uv = r.b_uv * S * Q;                   // >= E_u + E_v
    const float duv = ((e_uv + 2.0f * e_det) * KD + 8.0f * u0) * (1.0f + 4.0f * u0);
    // margins of half a triangle or more cull little: the caller tests the leaf in order instead
    lc.duv = duv;
    if (!(duv < max_duv)) return lc;
    const float R = 4.0f * (duv + 2.0f * u0) * Q * 1.0001f + 1e-30f;
    if (!(R < kCullHuge)) return lc;
    const float e_t = kCullSafety * 36.0f * u0 * S * P;
    // Dt(t) = (E_t + t E_det) / Dlo + 2 u0 t <= dt0 + t dt1
    lc.dt0 = e_t * KD * (1.0f + 4.0f * u0);
    lc.dt1 = (e_det * KD + 4.0f * u0) * (1.0f + 4.0f * u0);
    lc.thi = leaf_thi(lc, t_best);
    const float th = 0.0001f;  // the test's threshold (triangle.rs:47)
    lc.tlo = cull_down(th - (lc.dt0 + th * lc.dt1) * (1.0f + 8.0f * u0)) - 1e-30f;
    for (int i = 0; i < 3; ++i) {
        const float g = R + 8.0f * u0 * (2.0f * B + cull_abs(r.o[i]) + R) + 1e-30f;
        const float clo = r.o[i] + g, chi = r.o[i] - g;
        if (lc.zero & (1u << i)) {  // the line keeps o_i: culled when the grown slab does not contain it
            lc.slo[i] = clo;
            lc.shi[i] = chi;
        } else {                    // t = (lo - c_lo) / d = fma(lo, 1/d, -c_lo / d)
            lc.slo[i] = -(clo * r.rd[i]);
            lc.shi[i] = -(chi * r.rd[i]);
        }
    }
    lc.on = true;
    return lc;
}

// Whether the line of the ray, between lc.tlo and lc.thi, meets the box [lo, hi] grown by the
// leaf's margins (always true when !lc.on); t_enter: where it enters (for near-first order).
BVHGPU_HD bool box_live(const float lo[3], const float hi[3], const float rd[3], const LeafCull& lc, float& t_enter) {
    t_enter = 0.0f;
    if (!lc.on) return true;
    float tlo = lc.tlo, thi = lc.thi;
    bool out = false;
    for (int i = 0; i < 3; ++i) {
        if (lc.zero & (1u << i)) {
            out = out || lo[i] > lc.slo[i] || hi[i] < lc.shi[i];
        } else {
            const float t1 = cull_fma(lo[i], rd[i], lc.slo[i]);
            const float t2 = cull_fma(hi[i], rd[i], lc.shi[i]);
            tlo = cull_fmax(tlo, cull_fmin(t1, t2));
            thi = cull_fmin(thi, cull_fmax(t1, t2));
        }
    }
    t_enter = tlo;
    return !out && !(tlo > thi);
}

}  // namespace bvhgpu
