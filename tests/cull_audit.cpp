// CPU audit of the library's exact cull (bvhtracer_gb300/csrc/cull.cuh), run by test_cull_audit.py.
//
// For random and adversarial (ray, group of 64 triangles) pairs -- rays aimed at edges and
// vertices, grazing the triangles' plane, axis-aligned, starting next to the surface; groups of
// random, sliver, nearly flat and flipped-winding triangles over seven orders of magnitude of
// scale -- a group whose box the cull rejects must contain no triangle that the reference's float
// Moeller-Trumbore test (triangle.rs:42-72, restated below, unfused) accepts at or below t_best.
// The normal-cone bound is also checked directly: it never exceeds the exact |d . (e1 x e2)| of
// any triangle of the group.  Usage: cull_audit <iterations per thread> [nmin scale]; a scale
// above 1 overclaims the cone bound on purpose (the sensitivity check must then fail).
#include <cstdio>
#include <cstdint>
#include <cmath>
#include <cfloat>
#include <random>
#include <thread>
#include <vector>
#include <atomic>
#include <algorithm>
#include "cull.cuh"
using namespace bvhgpu;

struct V { float x, y, z; };
static inline V sub(V a, V b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline V cross(V a, V b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
static inline float dot(V a, V b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
// the reference's test (triangle.rs:42-72), float, unfused (-ffp-contract=off)
static bool mt(V v0, V v1, V v2, V o, V d, float* t_out) {
    V e1 = sub(v1, v0), e2 = sub(v2, v0);
    V n = cross(d, e2);
    float a = dot(e1, n);
    if (std::fabs(a) < 0.0001f) return false;
    float f = 1.0f / a;
    V s = sub(o, v0);
    float u = f * dot(s, n);
    if (u < 0.0f || u > 1.0f) return false;
    V q = cross(s, e1);
    float v = f * dot(d, q);
    if (v < 0.0f || u + v > 1.0f) return false;
    float t = f * dot(e2, q);
    if (t > 0.0001f) { *t_out = t; return true; }
    return false;
}

int main(int argc, char** argv) {
    const int nthreads = 8;
    const long per_thread = argc > 1 ? atol(argv[1]) : 200000;
    const float nmin_scale = argc > 2 ? (float)atof(argv[2]) : 1.0f;
    std::atomic<long> violations{0}, culled{0}, pairs{0}, accepted_total{0}, coned{0}, cone_checked{0}, cone_bad{0};
    std::atomic<double> cone_ratio_max{0.0};
    std::vector<std::thread> th;
    for (int w = 0; w < nthreads; ++w) th.emplace_back([&, w] {
        std::mt19937_64 rng(1234 + w);
        std::uniform_real_distribution<double> U(0.0, 1.0);
        auto urand = [&](double a, double b) { return (float)(a + (b - a) * U(rng)); };
        for (long it = 0; it < per_thread; ++it) {
            // cluster: 64 triangles, scale and shape vary
            const int kind = (int)(U(rng) * 6);
            const double scale = std::pow(10.0, urand(-2.5, 3.5));
            const double size = scale * std::pow(10.0, urand(-3, 0));
            V center = {urand(-1, 1) * (float)scale, urand(-1, 1) * (float)scale, urand(-1, 1) * (float)scale};
            V tv[64][3];
            for (int k = 0; k < 64; ++k) {
                V p = {center.x + urand(-1, 1) * (float)size, center.y + urand(-1, 1) * (float)size,
                       center.z + urand(-1, 1) * (float)size};
                double es = size * (kind == 0 ? 0.05 : (kind == 1 ? 0.5 : (kind == 2 ? 1e-3 : 2.0)));
                V a = {p.x + urand(-1, 1) * (float)es, p.y + urand(-1, 1) * (float)es, p.z + urand(-1, 1) * (float)es};
                V b = {p.x + urand(-1, 1) * (float)es, p.y + urand(-1, 1) * (float)es, p.z + urand(-1, 1) * (float)es};
                if (kind == 3 && k % 2) b = {a.x + (p.x - a.x) * 1e-3f, a.y + (p.y - a.y) * 1e-3f, p.z};  // slivers
                if (kind >= 4) {  // a bumpy patch of the plane z = cz: normals within a narrow cone
                    const float es2 = (float)(size * 0.1);
                    const float bump = (float)(size * 0.01) * urand(0, 1);
                    p.z = center.z + bump * urand(-1, 1);
                    a = {p.x + es2, p.y + urand(-0.2f, 0.2f) * es2, center.z + bump * urand(-1, 1)};
                    b = {p.x + urand(-0.2f, 0.2f) * es2, p.y + es2, center.z + bump * urand(-1, 1)};
                    if (kind == 5 && k % 2) std::swap(a, b);  // flipped winding
                }
                tv[k][0] = p; tv[k][1] = a; tv[k][2] = b;
            }
            float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
            float e1m = 0, e2m = 0;
            for (int k = 0; k < 64; ++k) {
                V e1 = sub(tv[k][1], tv[k][0]), e2 = sub(tv[k][2], tv[k][0]);
                V p1 = {tv[k][0].x + e1.x, tv[k][0].y + e1.y, tv[k][0].z + e1.z};
                V p2 = {tv[k][0].x + e2.x, tv[k][0].y + e2.y, tv[k][0].z + e2.z};
                V pts[3] = {tv[k][0], p1, p2};
                for (int j = 0; j < 3; ++j) {
                    const float* pv = &pts[j].x;
                    for (int i = 0; i < 3; ++i) { lo[i] = std::min(lo[i], pv[i]); hi[i] = std::max(hi[i], pv[i]); }
                }
                e1m = std::max({e1m, std::fabs(e1.x), std::fabs(e1.y), std::fabs(e1.z)});
                e2m = std::max({e2m, std::fabs(e2.x), std::fabs(e2.y), std::fabs(e2.z)});
            }
            GroupSeal c = group_seal(lo, hi, e1m, e2m, true);
            // the cluster's normal cone: axis = sum of unit normals, then the bounds
            double sx = 0, sy = 0, sz = 0;
            for (int k = 0; k < 64; ++k) {
                V e1 = sub(tv[k][1], tv[k][0]), e2 = sub(tv[k][2], tv[k][0]), nn = cross(e1, e2);
                double l = std::sqrt((double)nn.x * nn.x + (double)nn.y * nn.y + (double)nn.z * nn.z);
                if (l > 0) { double sg = (sx * nn.x + sy * nn.y + sz * nn.z) < 0 ? -1 : 1; sx += sg * nn.x / l; sy += sg * nn.y / l; sz += sg * nn.z / l; }
            }
            LeafCone cone{(float)sx, (float)sy, (float)sz, 2.0f, 0.0f, FLT_MAX};
            for (int k = 0; k < 64; ++k) {
                V e1 = sub(tv[k][1], tv[k][0]), e2 = sub(tv[k][2], tv[k][0]);
                float ca[3] = {e1.x, e1.y, e1.z}, cb[3] = {e2.x, e2.y, e2.z}, cl, nl;
                cone_terms(ca, cb, cone.ax, cone.ay, cone.az, cl, nl);
                cone.cos_phi = std::min(cone.cos_phi, cl);
                cone.nmin = std::min(cone.nmin, nl);
            }
            cone.sin_phi = cone_sin(cone.cos_phi);
            if (U(rng) < 0.1) cone.nmin = 0.0f;  // sometimes no cone at all
            cone.nmin *= nmin_scale;
            // rays: aimed at a point near a triangle's boundary (edge / vertex / interior), grazing, random
            for (int r = 0; r < 16; ++r) {
                const int k = (int)(U(rng) * 64);
                V A = tv[k][0], Bv = tv[k][1], C = tv[k][2];
                double a = U(rng), b = U(rng) * (1 - a);
                const int mode = (int)(U(rng) * 5);
                if (mode == 0) b = 0;                  // on an edge
                if (mode == 1) { a = 1; b = 0; }       // vertex
                if (mode == 2) { b = 1 - a; }          // hypotenuse
                const double over = std::pow(10.0, urand(-9, -1)) * (U(rng) < 0.5 ? -1 : 1);
                a += over; b += over * (U(rng) < 0.5 ? 1 : -1);
                V target = {(float)(A.x + a * (Bv.x - A.x) + b * (C.x - A.x)), (float)(A.y + a * (Bv.y - A.y) + b * (C.y - A.y)),
                            (float)(A.z + a * (Bv.z - A.z) + b * (C.z - A.z))};
                V dir;
                if (mode == 4) {  // grazing: along the triangle plane with a tiny normal part
                    V e1 = sub(Bv, A), e2 = sub(C, A), nn = cross(e1, e2);
                    float nl = std::sqrt(dot(nn, nn));
                    float el = std::sqrt(dot(e1, e1));
                    float g = (float)std::pow(10.0, urand(-7, -1));
                    dir = {e1.x / el + g * nn.x / nl, e1.y / el + g * nn.y / nl, e1.z / el + g * nn.z / nl};
                } else {
                    dir = {urand(-1, 1), urand(-1, 1), urand(-1, 1)};
                }
                float dl = std::sqrt(dot(dir, dir));
                if (!(dl > 0)) continue;
                dir = {dir.x / dl, dir.y / dl, dir.z / dl};
                const float back = U(rng) < 0.2 ? (float)(size * std::pow(10.0, urand(-7, -1))) : (float)(scale * std::pow(10.0, urand(-3, 1.5)));
                V o = {target.x - dir.x * back, target.y - dir.y * back, target.z - dir.z * back};
                // t_best: none, near the target distance, or random
                float tb = FLT_MAX;
                const double pick = U(rng);
                if (pick < 0.4) tb = back * (float)(1.0 + urand(-1e-3, 1e-3));
                else if (pick < 0.6) tb = back * urand(0.0, 2.0);
                pairs++;
                if (U(rng) < 0.15) { int ax = (int)(U(rng) * 3); (&dir.x)[ax] = 0.0f; if (U(rng) < 0.3) { o = {target.x - dir.x * back, target.y - dir.y * back, target.z - dir.z * back}; } }
                {
                    CullRay q0 = cull_ray(o.x, o.y, o.z, dir.x, dir.y, dir.z);
                    const float dlo = cone_det_lo(q0.d, cone);
                    if (dlo > 1e-4f) coned++;
                    // the cone bound itself: |d . (e1 x e2)| in exact arithmetic never below it
                    double worst = 1e300;
                    for (int q = 0; q < 64; ++q) {
                        V e1 = sub(tv[q][1], tv[q][0]), e2 = sub(tv[q][2], tv[q][0]);
                        double nx = (double)e1.y * e2.z - (double)e1.z * e2.y, ny = (double)e1.z * e2.x - (double)e1.x * e2.z,
                               nz = (double)e1.x * e2.y - (double)e1.y * e2.x;
                        double det = std::fabs(nx * dir.x + ny * dir.y + nz * dir.z);
                        worst = std::min(worst, det);
                    }
                    if (dlo > 0) {
                        cone_checked++;
                        cone_ratio_max = std::max(cone_ratio_max.load(), (double)dlo / worst);
                        if ((double)dlo > worst && cone_bad++ < 5) printf("CONE VIOLATION kind %d dlo %g worst %g\n", kind, dlo, worst);
                    }
                }
                LeafCull lc = leaf_cull(cull_ray(o.x, o.y, o.z, dir.x, dir.y, dir.z), c.q, c.b, tb, 1e30f, cone);
                float te; CullRay crr = cull_ray(o.x, o.y, o.z, dir.x, dir.y, dir.z); if (box_live(c.lo, c.hi, crr.rd, lc, te)) continue;
                culled++;
                for (int q = 0; q < 64; ++q) {
                    float t;
                    if (mt(tv[q][0], tv[q][1], tv[q][2], o, dir, &t) && t <= tb) {
                        if (violations++ < 10)
                            printf("VIOLATION kind %d mode %d tri %d t %g tb %g scale %g size %g cone %g %g\n", kind, mode, q, t, tb, scale, size, cone.cos_phi, cone.nmin);
                    }
                }
            }
            // also count accepted hits in general (the audit must see many near-boundary hits)
            float t;
            V o = {center.x, center.y, (float)(center.z - 3 * scale)}, d = {0, 0, 1};
            if (mt(tv[0][0], tv[0][1], tv[0][2], o, d, &t)) accepted_total++;
        }
    });
    for (auto& t : th) t.join();
    printf("pairs %ld culled %ld (%.1f%%) cone-tightened %ld violations %ld | cone bounds checked %ld, max(bound / min |det*|) %.4f, cone violations %ld\n", pairs.load(), culled.load(), 100.0 * culled.load() / pairs.load(), coned.load(), violations.load(), cone_checked.load(), cone_ratio_max.load(), cone_bad.load());
    return (violations.load() || cone_bad.load()) ? 1 : 0;
}
