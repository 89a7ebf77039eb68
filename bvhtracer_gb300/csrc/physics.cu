// Rigid-body physics driving instance transforms, on the device: World::run_physics
// (BT/src/physics/world.rs:56-59), RigidBody::integrate / calculate_derived_data
// (physics/rigid_body.rs:132-213), the Gravity and Spring force generators
// (physics/force_generator.rs:44-155) and SceneObject::update_transform (scene_object.rs:52-58),
// so that Scene::run (scene.rs:40-50) -- physics, transforms, TLAS rebuild -- is one device
// sequence that a frame graph can capture.
//
// Every step is written with explicit round-to-nearest operations in the reference's order
// (left-to-right sums).  Two things are not pinned bit for bit: powf (drag factors, and the sleep
// bias of bodies that can sleep) is a transcendental whose last bit differs between math
// libraries -- drag 1 and can_sleep false, the setting of the reference's demos, never reach it
// (powf(1, x) is exactly 1) -- and the quaternion product / norm and the 4x4 inverse of the
// reference's linear-algebra crate, which are restated from their textbook formulas.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <string>
#include <vector>

#include "common.cuh"
#include "internal.hpp"

namespace bvhgpu {
namespace {

typedef bvhgpu_rigid_body Body;

__device__ __forceinline__ void xf_point4(const float* m, const float* p, float* out) {  // M * (p, 1)
    for (int r = 0; r < 3; ++r)
        out[r] = fadd(fadd(fadd(fmul(m[r], p[0]), fmul(m[4 + r], p[1])), fmul(m[8 + r], p[2])), fmul(m[12 + r], 1.0f));
}
__device__ __forceinline__ float mag3(const float* v) {
    return __fsqrt_rn(fadd(fadd(fmul(v[0], v[0]), fmul(v[1], v[1])), fmul(v[2], v[2])));
}

// RigidBody::apply_force_at_point (rigid_body.rs:434-440)
__device__ __forceinline__ void apply_force_at_point(Body& b, const float* f, const float* p) {
    const float cm[3] = {fsub(p[0], b.position[0]), fsub(p[1], b.position[1]), fsub(p[2], b.position[2])};
    for (int k = 0; k < 3; ++k) b.force_accum[k] = fadd(b.force_accum[k], f[k]);
    const float t[3] = {fsub(fmul(cm[1], f[2]), fmul(cm[2], f[1])), fsub(fmul(cm[2], f[0]), fmul(cm[0], f[2])),
                        fsub(fmul(cm[0], f[1]), fmul(cm[1], f[0]))};
    for (int k = 0; k < 3; ++k) b.torque_accum[k] = fadd(b.torque_accum[k], t[k]);
    b.is_awake = 1u;
}

// ForceRegistry::apply_forces (force_registry.rs:73-77): each body's generators in registry order.
// A spring reads the other body's transform, which no force application changes.
__global__ void k_apply_forces(Body* bodies, uint32_t n, const bvhgpu_force_generator* __restrict__ gens,
                               const uint32_t* __restrict__ off) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Body& b = bodies[i];
    for (uint32_t g = off[i]; g < off[i + 1]; ++g) {
        const bvhgpu_force_generator& G = gens[g];
        if (G.kind == BVHGPU_FORCE_GRAVITY) {  // Gravity::apply_force (force_generator.rs:52-59)
            if (b.inverse_mass >= 0.0f) {
                const float mass = b.inverse_mass == 0.0f ? FLT_MAX : __fdiv_rn(1.0f, b.inverse_mass);
                for (int k = 0; k < 3; ++k) b.force_accum[k] = fadd(b.force_accum[k], fmul(G.gravity[k], mass));
                b.is_awake = 1u;
            }
        } else {  // Spring::apply_force (force_generator.rs:133-154)
            float lws[3], ows[3];
            xf_point4(b.transform, G.spring_point, lws);
            xf_point4(bodies[G.other].transform, G.other_point, ows);
            const float d[3] = {fsub(lws[0], ows[0]), fsub(lws[1], ows[1]), fsub(lws[2], ows[2])};
            const float len = mag3(d);
            const float fm = fmul(G.spring_constant, fabsf(fsub(len, G.rest_length)));
            const float m = mag3(d);  // normalize() takes its own magnitude
            const float f[3] = {fmul(__fdiv_rn(d[0], m), -fm), fmul(__fdiv_rn(d[1], m), -fm),
                                fmul(__fdiv_rn(d[2], m), -fm)};
            apply_force_at_point(b, f, lws);
        }
    }
}

// RigidBody::calculate_derived_data (rigid_body.rs:132-146): normalized orientation, the
// transform of Transform3::from_translation_rotation (transform.rs:190-217), the world-space
// inverse inertia tensor of _transform_inertia_tensor (rigid_body.rs:30-70).
__device__ void derived_data(Body& b) {
    float* q = b.orientation;
    const float m = __fsqrt_rn(fadd(fadd(fadd(fmul(q[0], q[0]), fmul(q[1], q[1])), fmul(q[2], q[2])),
                                    fmul(q[3], q[3])));
    for (int k = 0; k < 4; ++k) q[k] = __fdiv_rn(q[k], m);
    const float s = q[0], x = q[1], y = q[2], z = q[3], two = fadd(1.0f, 1.0f);
    float* M = b.transform;
    M[0] = fsub(fsub(1.0f, fmul(fmul(two, y), y)), fmul(fmul(two, z), z));
    M[1] = fadd(fmul(fmul(two, x), y), fmul(fmul(two, s), z));
    M[2] = fsub(fmul(fmul(two, x), z), fmul(fmul(two, s), y));
    M[3] = 0.0f;
    M[4] = fsub(fmul(fmul(two, x), y), fmul(fmul(two, s), z));
    M[5] = fsub(fsub(1.0f, fmul(fmul(two, x), x)), fmul(fmul(two, z), z));
    M[6] = fadd(fmul(fmul(two, y), z), fmul(fmul(two, s), x));
    M[7] = 0.0f;
    M[8] = fadd(fmul(fmul(two, x), z), fmul(fmul(two, s), y));
    M[9] = fsub(fmul(fmul(two, y), z), fmul(fmul(two, s), x));
    M[10] = fsub(fsub(1.0f, fmul(fmul(two, x), x)), fmul(fmul(two, y), y));
    M[11] = 0.0f;
    M[12] = b.position[0];
    M[13] = b.position[1];
    M[14] = b.position[2];
    M[15] = 1.0f;
    // iit_body[c][r] = I[3c + r]; rot_mat[c][r] = M[4c + r]
    const float* I = b.inverse_inertia;
    auto R = [&](int c, int r) { return M[4 * c + r]; };
    auto B = [&](int c, int r) { return I[3 * c + r]; };
    float t[3][3];  // t[a][k] = m_ka of the reference (m00, m10, m20, m01, ...)
    for (int a = 0; a < 3; ++a)
        for (int k = 0; k < 3; ++k)
            t[a][k] = fadd(fadd(fmul(R(0, a), B(k, 0)), fmul(R(1, a), B(k, 1))), fmul(R(2, a), B(k, 2)));
    float* W = b.inverse_inertia_world;
    for (int a = 0; a < 3; ++a)      // iit_world[c][a] for c = 0..2
        for (int c = 0; c < 3; ++c)
            W[3 * c + a] = fadd(fadd(fmul(t[a][0], R(0, c)), fmul(t[a][1], R(1, c))), fmul(t[a][2], R(2, c)));
}

__global__ void k_start_frame(Body* bodies, uint32_t n) {  // World::start_frame (world.rs:43-48)
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Body& b = bodies[i];
    for (int k = 0; k < 3; ++k) b.force_accum[k] = b.torque_accum[k] = 0.0f;
    derived_data(b);
}

// RigidBody::integrate (rigid_body.rs:149-213)
__global__ void k_integrate(Body* bodies, uint32_t n, float d) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Body& b = bodies[i];
    if (!b.is_awake) return;
    for (int k = 0; k < 3; ++k)
        b.last_frame_acceleration[k] = fadd(b.acceleration[k], fmul(b.force_accum[k], b.inverse_mass));
    const float* W = b.inverse_inertia_world;
    float aa[3];
    for (int r = 0; r < 3; ++r)
        aa[r] = fadd(fadd(fmul(W[r], b.torque_accum[0]), fmul(W[3 + r], b.torque_accum[1])),
                     fmul(W[6 + r], b.torque_accum[2]));
    for (int k = 0; k < 3; ++k) {
        b.velocity[k] = fadd(b.velocity[k], fmul(b.last_frame_acceleration[k], d));
        b.rotation[k] = fadd(b.rotation[k], fmul(aa[k], d));
    }
    const float ld = powf(b.linear_drag, d), ad = powf(b.angular_drag, d);
    for (int k = 0; k < 3; ++k) {
        b.velocity[k] = fmul(b.velocity[k], ld);
        b.rotation[k] = fmul(b.rotation[k], ad);
    }
    for (int k = 0; k < 3; ++k) b.position[k] = fadd(b.position[k], fmul(b.velocity[k], d));
    // q = (0, rotation * d) * orientation, orientation += q / 2
    const float px = fmul(b.rotation[0], d), py = fmul(b.rotation[1], d), pz = fmul(b.rotation[2], d);
    float* o = b.orientation;
    const float s2 = o[0], x2 = o[1], y2 = o[2], z2 = o[3];
    const float qs = fsub(fsub(fsub(fmul(0.0f, s2), fmul(px, x2)), fmul(py, y2)), fmul(pz, z2));
    const float qx = fsub(fadd(fadd(fmul(0.0f, x2), fmul(px, s2)), fmul(py, z2)), fmul(pz, y2));
    const float qy = fadd(fadd(fsub(fmul(0.0f, y2), fmul(px, z2)), fmul(py, s2)), fmul(pz, x2));
    const float qz = fadd(fsub(fadd(fmul(0.0f, z2), fmul(px, y2)), fmul(py, x2)), fmul(pz, s2));
    o[0] = fadd(o[0], fmul(qs, 0.5f));
    o[1] = fadd(o[1], fmul(qx, 0.5f));
    o[2] = fadd(o[2], fmul(qy, 0.5f));
    o[3] = fadd(o[3], fmul(qz, 0.5f));
    derived_data(b);
    for (int k = 0; k < 3; ++k) b.force_accum[k] = b.torque_accum[k] = 0.0f;
    if (b.can_sleep) {
        const float* v = b.velocity;
        const float* r = b.rotation;
        const float cur = fadd(fadd(fadd(fmul(v[0], v[0]), fmul(v[1], v[1])), fmul(v[2], v[2])),
                               fadd(fadd(fmul(r[0], r[0]), fmul(r[1], r[1])), fmul(r[2], r[2])));
        const float bias = powf(0.5f, d);
        b.motion = fadd(fmul(bias, b.motion), fmul(fsub(1.0f, bias), cur));
        const float thr = 0.3f, cap = fmul(10.0f, 0.3f);
        if (b.motion < thr) {  // set_awake(false)
            b.is_awake = 0u;
            for (int k = 0; k < 3; ++k) b.velocity[k] = b.rotation[k] = 0.0f;
        } else if (b.motion > cap) {
            b.motion = cap;
        }
    }
}

// 4x4 inverse by cofactors (column-major): inv = adj(M) / det(M); det by the first column.
__device__ void inverse4(const float* m, float* out) {
    auto e = [&](int r, int c) { return m[4 * c + r]; };
    float cof[16];
    for (int r = 0; r < 4; ++r) {
        for (int c = 0; c < 4; ++c) {
            int rr[3], cc[3];
            for (int k = 0, j = 0; k < 4; ++k)
                if (k != r) rr[j++] = k;
            for (int k = 0, j = 0; k < 4; ++k)
                if (k != c) cc[j++] = k;
            const float d3 = fadd(fsub(fmul(e(rr[0], cc[0]), fsub(fmul(e(rr[1], cc[1]), e(rr[2], cc[2])),
                                                                  fmul(e(rr[1], cc[2]), e(rr[2], cc[1])))),
                                       fmul(e(rr[0], cc[1]), fsub(fmul(e(rr[1], cc[0]), e(rr[2], cc[2])),
                                                                  fmul(e(rr[1], cc[2]), e(rr[2], cc[0]))))),
                                  fmul(e(rr[0], cc[2]), fsub(fmul(e(rr[1], cc[0]), e(rr[2], cc[1])),
                                                             fmul(e(rr[1], cc[1]), e(rr[2], cc[0])))));
            cof[4 * r + c] = ((r + c) & 1) ? -d3 : d3;
        }
    }
    const float det = fadd(fadd(fadd(fmul(e(0, 0), cof[0]), fmul(e(1, 0), cof[4])), fmul(e(2, 0), cof[8])),
                           fmul(e(3, 0), cof[12]));
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) out[4 * c + r] = __fdiv_rn(cof[4 * c + r], det);  // adj = cof^T
}

// SceneObject::update_transform (scene_object.rs:52-58): body transform * initial transform, and
// the cached inverse of TransformComponent3::set_transform (transform_component.rs:24-27).
__global__ void k_update_from_bodies(const Body* __restrict__ bodies, const uint32_t* __restrict__ body_of,
                                     const float* __restrict__ init, uint32_t nobj, float* xf, float* inv) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nobj) return;
    const uint32_t bi = body_of[i];
    if (bi == 0xFFFFFFFFu) return;
    const float* A = bodies[bi].transform;
    const float* B = init + 16ull * i;
    float P[16];
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r)
            P[4 * c + r] = fadd(fadd(fadd(fmul(A[r], B[4 * c]), fmul(A[4 + r], B[4 * c + 1])),
                                     fmul(A[8 + r], B[4 * c + 2])),
                                fmul(A[12 + r], B[4 * c + 3]));
    float Q[16];
    inverse4(P, Q);
    for (int k = 0; k < 16; ++k) {
        xf[16ull * i + k] = P[k];
        inv[16ull * i + k] = Q[k];
    }
}

inline unsigned grid_of(uint32_t n) { return (n + 127) / 128; }

}  // namespace

cudaError_t launch_world_start_frame(bvhgpu_ctx* ctx, DeviceWorld& w, cudaStream_t s) {
    if (w.nbodies == 0) return cudaSuccess;
    LaunchScope scope(ctx, BVHGPU_K_OTHER, s);
    k_start_frame<<<grid_of(w.nbodies), 128, 0, s>>>(w.bodies, w.nbodies);
    g_launches++;
    return cudaGetLastError();
}

cudaError_t launch_world_step(bvhgpu_ctx* ctx, DeviceWorld& w, float dt, cudaStream_t s) {
    if (w.nbodies == 0) return cudaSuccess;
    LaunchScope scope(ctx, BVHGPU_K_OTHER, s);
    k_apply_forces<<<grid_of(w.nbodies), 128, 0, s>>>(w.bodies, w.nbodies, w.gens, w.gen_off);
    k_integrate<<<grid_of(w.nbodies), 128, 0, s>>>(w.bodies, w.nbodies, dt);
    g_launches += 2;
    return cudaGetLastError();
}

cudaError_t launch_update_from_bodies(bvhgpu_ctx* ctx, DeviceScene& sc, const DeviceWorld& w, cudaStream_t s) {
    LaunchScope scope(ctx, BVHGPU_K_OTHER, s);
    k_update_from_bodies<<<grid_of(sc.nobjects), 128, 0, s>>>(w.bodies, sc.body_of, sc.transform_init, sc.nobjects,
                                                              sc.xf, sc.inv);
    g_launches++;
    return cudaGetLastError();
}

}  // namespace bvhgpu

// ---- C ABI ----------------------------------------------------------------------------------------

using namespace bvhgpu;

namespace {

int phys_fail(bvhgpu_ctx* ctx, int code, const char* what) { return record_error(ctx, code, what); }

int phys_cuda(bvhgpu_ctx* ctx, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return BVHGPU_OK;
    std::string msg = std::string(what) + ": " + cudaGetErrorString(e);
    return record_error(ctx, BVHGPU_ERR_CUDA, msg.c_str());
}

cudaStream_t phys_stream(bvhgpu_ctx* ctx, bvhgpu_stream s) { return s ? static_cast<cudaStream_t>(s) : ctx->stream; }

void free_world(DeviceWorld& w) {
    cudaFree(w.bodies);
    cudaFree(w.gens);
    cudaFree(w.gen_off);
    w = DeviceWorld{};
}

}  // namespace

void bvhgpu_free_worlds(bvhgpu_ctx* ctx) {
    for (auto& kv : ctx->worlds) free_world(kv.second);
    ctx->worlds.clear();
}

extern "C" {

int bvhgpu_world_create(bvhgpu_ctx* ctx, const bvhgpu_rigid_body* bodies, uint32_t nbodies,
                        const bvhgpu_force_generator* gens, uint32_t ngens, uint32_t* world_id) {
    if (!ctx || !world_id || (nbodies && !bodies) || (ngens && !gens)) return BVHGPU_ERR_INVALID_ARG;
    for (uint32_t g = 0; g < ngens; ++g) {
        if (gens[g].body >= nbodies || (gens[g].kind == BVHGPU_FORCE_SPRING && gens[g].other >= nbodies) ||
            gens[g].kind > BVHGPU_FORCE_SPRING)
            return phys_fail(ctx, BVHGPU_ERR_INVALID_ARG, "world_create: bad force generator");
    }
    // group the registry by body, registry order kept within each body
    std::vector<uint32_t> off(nbodies + 1, 0);
    for (uint32_t g = 0; g < ngens; ++g) off[gens[g].body + 1]++;
    for (uint32_t i = 0; i < nbodies; ++i) off[i + 1] += off[i];
    std::vector<bvhgpu_force_generator> grouped(ngens);
    std::vector<uint32_t> fill(off.begin(), off.end() - 1);
    for (uint32_t g = 0; g < ngens; ++g) grouped[fill[gens[g].body]++] = gens[g];
    DeviceWorld w;
    w.nbodies = nbodies;
    w.ngens = ngens;
    cudaError_t e = cudaMalloc(&w.bodies, sizeof(bvhgpu_rigid_body) * std::max<uint32_t>(nbodies, 1));
    if (e == cudaSuccess) e = cudaMalloc(&w.gens, sizeof(bvhgpu_force_generator) * std::max<uint32_t>(ngens, 1));
    if (e == cudaSuccess) e = cudaMalloc(&w.gen_off, sizeof(uint32_t) * (nbodies + 1));
    if (e == cudaSuccess && nbodies)
        e = cudaMemcpy(w.bodies, bodies, sizeof(bvhgpu_rigid_body) * nbodies, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && ngens)
        e = cudaMemcpy(w.gens, grouped.data(), sizeof(bvhgpu_force_generator) * ngens, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(w.gen_off, off.data(), sizeof(uint32_t) * (nbodies + 1), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        free_world(w);
        return phys_cuda(ctx, e, "world_create");
    }
    *world_id = ctx->next_world++;
    ctx->worlds[*world_id] = w;
    return BVHGPU_OK;
}

int bvhgpu_world_free(bvhgpu_ctx* ctx, uint32_t world_id) {
    if (!ctx) return BVHGPU_ERR_INVALID_ARG;
    auto it = ctx->worlds.find(world_id);
    if (it == ctx->worlds.end()) return phys_fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown world");
    cudaStreamSynchronize(ctx->stream);
    for (auto& kv : ctx->scenes)
        if (kv.second.world == world_id) kv.second.world = 0;
    free_world(it->second);
    ctx->worlds.erase(it);
    return BVHGPU_OK;
}

int bvhgpu_world_start_frame_async(bvhgpu_ctx* ctx, uint32_t world_id, bvhgpu_stream s) {
    if (!ctx) return BVHGPU_ERR_INVALID_ARG;
    auto it = ctx->worlds.find(world_id);
    if (it == ctx->worlds.end()) return phys_fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown world");
    return phys_cuda(ctx, launch_world_start_frame(ctx, it->second, phys_stream(ctx, s)), "world start frame");
}

int bvhgpu_world_step_async(bvhgpu_ctx* ctx, uint32_t world_id, float dt, bvhgpu_stream s) {
    if (!ctx) return BVHGPU_ERR_INVALID_ARG;
    auto it = ctx->worlds.find(world_id);
    if (it == ctx->worlds.end()) return phys_fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown world");
    return phys_cuda(ctx, launch_world_step(ctx, it->second, dt, phys_stream(ctx, s)), "world step");
}

int bvhgpu_world_download(bvhgpu_ctx* ctx, uint32_t world_id, bvhgpu_rigid_body* bodies_out) {
    if (!ctx || !bodies_out) return BVHGPU_ERR_INVALID_ARG;
    auto it = ctx->worlds.find(world_id);
    if (it == ctx->worlds.end()) return phys_fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown world");
    int rc = phys_cuda(ctx, cudaStreamSynchronize(ctx->stream), "stream synchronize");
    if (rc) return rc;
    return phys_cuda(ctx, cudaMemcpy(bodies_out, it->second.bodies, sizeof(bvhgpu_rigid_body) * it->second.nbodies,
                                     cudaMemcpyDeviceToHost),
                     "download bodies");
}

int bvhgpu_scene_bind_world(bvhgpu_ctx* ctx, uint32_t scene_id, uint32_t world_id, const uint32_t* body_of,
                            const float* transform_init) {
    if (!ctx || !body_of || !transform_init) return BVHGPU_ERR_INVALID_ARG;
    auto sc = ctx->scenes.find(scene_id);
    auto w = ctx->worlds.find(world_id);
    if (sc == ctx->scenes.end() || w == ctx->worlds.end())
        return phys_fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown scene or world");
    DeviceScene& S = sc->second;
    for (uint32_t i = 0; i < S.nobjects; ++i)
        if (body_of[i] != 0xFFFFFFFFu && body_of[i] >= w->second.nbodies)
            return phys_fail(ctx, BVHGPU_ERR_INVALID_ARG, "scene_bind_world: body index out of range");
    cudaStreamSynchronize(ctx->stream);
    if (!S.body_of && cudaMalloc(&S.body_of, 4ull * std::max<uint32_t>(S.nobjects, 1)) != cudaSuccess)
        return phys_fail(ctx, BVHGPU_ERR_OUT_OF_MEMORY, "scene_bind_world");
    if (!S.transform_init && cudaMalloc(&S.transform_init, 64ull * std::max<uint32_t>(S.nobjects, 1)) != cudaSuccess)
        return phys_fail(ctx, BVHGPU_ERR_OUT_OF_MEMORY, "scene_bind_world");
    cudaError_t e = cudaMemcpy(S.body_of, body_of, 4ull * S.nobjects, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(S.transform_init, transform_init, 64ull * S.nobjects, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return phys_cuda(ctx, e, "scene_bind_world");
    S.world = world_id;
    return BVHGPU_OK;
}

int bvhgpu_scene_run_async(bvhgpu_ctx* ctx, uint32_t scene_id, float dt, bvhgpu_stream s) {
    if (!ctx) return BVHGPU_ERR_INVALID_ARG;
    auto sc = ctx->scenes.find(scene_id);
    if (sc == ctx->scenes.end()) return phys_fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown scene");
    DeviceScene& S = sc->second;
    auto w = ctx->worlds.find(S.world);
    if (w == ctx->worlds.end()) return phys_fail(ctx, BVHGPU_ERR_INVALID_ARG, "scene has no bound world");
    const cudaStream_t st = phys_stream(ctx, s);
    int rc = phys_cuda(ctx, launch_world_step(ctx, w->second, dt, st), "world step");
    if (!rc) rc = phys_cuda(ctx, launch_update_from_bodies(ctx, S, w->second, st), "update transforms");
    if (rc) return rc;
    return bvhgpu_scene_rebuild_async(ctx, scene_id, s);
}

}  // extern "C"
