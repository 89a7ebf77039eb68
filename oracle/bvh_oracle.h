/*
 * CPU oracle for the ray-BVH hot path of lambdaxymox/bvhtracer.
 *
 * TEST INFRASTRUCTURE ONLY.  This is an operation-for-operation restatement of
 * the reference's Rust code (file:line citations beside each function in
 * bvh_oracle.cpp).  It exists to check the CUDA library and to be timed as the
 * CPU baseline; the product library never links, loads or calls it.
 *
 * The reference itself cannot be compiled in this environment (it is Rust and
 * no cargo/rustc is available), so this restatement is pinned against the
 * known answers asserted in the reference's own tests (exact f32 hit distances,
 * primitive ids of the cube scene, the 640x640 quad visibility mask, refit
 * identity / idempotence, node-array invariants).
 *
 * Build: see oracle/Makefile (-O2 -ffp-contract=off -fno-fast-math).
 */
#ifndef BVH_ORACLE_H
#define BVH_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same memory layouts as the product ABI (include/bvhgpu.h). */
typedef struct { float bounds_min[3]; float bounds_max[3]; uint32_t primitive_count; uint32_t left_first; } orc_node;
typedef struct { float v[9]; } orc_tri;
typedef struct { float origin[3]; float t; float direction[3]; uint32_t pad; } orc_ray;
typedef struct { float t, u, v; uint32_t prim, inst; } orc_hit;
typedef struct { float bounds_min[3]; float bounds_max[3]; uint32_t left_right; uint32_t blas; } orc_tlas_node;
/* Per-ray work counters (same traversal order as the reference). */
typedef struct { uint32_t interior; uint32_t leaves; uint32_t tris; uint32_t tlas_interior; uint32_t blas_entries; } orc_counters;

#define ORC_OK 0
#define ORC_ERR_ARG 1
#define ORC_ERR_PANIC 2   /* the reference would panic on this input */

/* --- primitives ---------------------------------------------------------- */
int orc_triangle_intersect(const orc_tri* tri, const orc_ray* ray, float* t, float* u, float* v);
int orc_aabb_intersect(const float bmin[3], const float bmax[3], const orc_ray* ray, float* tmin);
void orc_normalize(const float in[3], float out[3]);
void orc_triangle_centroid(const orc_tri* tri, float out[3]);

/* --- BLAS ----------------------------------------------------------------- */
/* BvhBuilder::build_for.  Reorders mesh in place; nodes_out has room for 2n nodes. */
int orc_bvh_build(orc_tri* mesh, uint32_t n, orc_node* nodes_out, uint32_t* nodes_used);
/* Bvh::intersect for a batch of rays (single thread).  counters may be NULL. */
int orc_bvh_intersect(const orc_node* nodes, uint32_t nodes_used, const orc_tri* mesh, uint32_t n,
                      const orc_ray* rays, uint32_t nrays, orc_hit* hits, orc_counters* counters);
/* Same, split over nthreads host threads. */
/* Every ray against a triangle list: mode 0 Triangle::intersect (first smallest t), mode 1
 * Triangle::intersect_mut on one Intersection per ray. */
int orc_triangles_intersect(const orc_tri* mesh, uint32_t ntris, const orc_ray* rays, uint32_t nrays, int mode,
                            orc_hit* hits);
/* Rigid bodies (BT/src/physics/rigid_body.rs) and force generators (force_generator.rs); the same
 * layout as the library's bvhgpu_rigid_body / bvhgpu_force_generator. */
typedef struct {
    float inverse_mass;
    float inverse_inertia[9];
    float linear_drag, angular_drag;
    float position[3];
    float orientation[4];
    float velocity[3];
    float rotation[3];
    float inverse_inertia_world[9];
    float motion;
    uint32_t is_awake, can_sleep;
    float transform[16];
    float force_accum[3], torque_accum[3];
    float acceleration[3], last_frame_acceleration[3];
} orc_rigid_body;
typedef struct {
    uint32_t kind, body, other, reserved;
    float gravity[3];
    float spring_point[3];
    float other_point[3];
    float spring_constant, rest_length;
} orc_force_generator;
/* World::start_frame, World::run_physics(dt) (registry order), SceneObject::update_transform. */
int orc_world_start_frame(orc_rigid_body* bodies, uint32_t n);
int orc_world_step(orc_rigid_body* bodies, uint32_t n, const orc_force_generator* gens, uint32_t ngens, float dt);
int orc_object_transforms(const orc_rigid_body* bodies, const uint32_t* body_of, const float* init, uint32_t nobj,
                          float* xf, float* inv);
/* Two smallest hit distances per ray over the whole BVH (FLT_MAX where there is none). */
int orc_two_nearest_mt(const orc_node* nodes, const orc_tri* mesh, const orc_ray* rays, uint32_t nrays, float* t1,
                       float* t2, int nthreads);
int orc_bvh_intersect_mt(const orc_node* nodes, uint32_t nodes_used, const orc_tri* mesh, uint32_t n,
                         const orc_ray* rays, uint32_t nrays, orc_hit* hits, int nthreads);
/* Bvh::refit, in place. */
int orc_bvh_refit(orc_node* nodes, uint32_t nodes_used, const orc_tri* mesh, uint32_t n);
/* Maximum depth of the tree (root = 1). */
uint32_t orc_bvh_depth(const orc_node* nodes, uint32_t nodes_used);

/* --- TLAS / scene ------------------------------------------------------------ */
/* SceneObject::set_transform: world bounds of the 8 transformed corners. */
void orc_object_bounds(const float model_min[3], const float model_max[3], const float xf[16],
                       float out_min[3], float out_max[3]);
/* TlasBuilder::build_for / Tlas::rebuild over per-object world bounds.
 * nodes_out has room for 2*count nodes. */
int orc_tlas_build(const float* obj_min, const float* obj_max, uint32_t count, orc_tlas_node* nodes_out,
                   uint32_t* nodes_used);
/* Scene::intersect.  For object i: blas_of[i] selects a BLAS; inv is 16 floats per object
 * (column-major, the cached inverse transform).  BLAS arrays are concatenated:
 * node_off[b], tri_off[b] give the first node / triangle of BLAS b. */
int orc_scene_intersect(const orc_tlas_node* tlas, uint32_t tlas_nodes_used,
                        const uint32_t* blas_of, const float* inv, uint32_t nobj,
                        const orc_node* nodes, const uint32_t* node_off,
                        const orc_tri* tris, const uint32_t* tri_off,
                        const orc_ray* rays, uint32_t nrays, orc_hit* hits, orc_counters* counters,
                        int reference_instance_zero);
int orc_scene_intersect_mt(const orc_tlas_node* tlas, uint32_t tlas_nodes_used,
                           const uint32_t* blas_of, const float* inv, uint32_t nobj,
                           const orc_node* nodes, const uint32_t* node_off,
                           const orc_tri* tris, const uint32_t* tri_off,
                           const orc_ray* rays, uint32_t nrays, orc_hit* hits, int nthreads);

/* --- camera / renderer -------------------------------------------------------- */
/* Camera::get_ray_world.  corners = top_left, top_right, bottom_left (eye space, 9 floats);
 * view_inv = 16 floats column-major. */
void orc_camera_ray(const float corners[9], const float view_inv[16], float u, float v, orc_ray* out);
/* PathTracer::evaluate over a w x h frame (8x8 tiles, pixel top-left corner samples) on a
 * single BLAS; accumulator / shader kinds as in include/bvhgpu.h. */
int orc_render_textured(const float corners[9], const float view_inv[16], int width, int height, int accumulator,
                        const float* acc_params, int shader, const float* shader_params, const orc_node* nodes,
                        uint32_t nodes_used, const orc_tri* tris, uint32_t ntris, const float* normals,
                        const float* tex_coords, const uint8_t* texels, uint32_t tex_w, uint32_t tex_h,
                        uint8_t* rgba, float* radiance);
int orc_render(const float corners[9], const float view_inv[16], int width, int height,
               int accumulator, const float* acc_params, int shader, const float* shader_params,
               const orc_node* nodes, uint32_t nodes_used, const orc_tri* tris, uint32_t ntris,
               const float* normals /* 9 floats per triangle, may be NULL */,
               uint8_t* rgba, float* radiance);

/* PathTracer::evaluate over a Scene (the TLAS with instance transforms).  lookup 0: the normal /
 * texture accumulators read object 0's model and transform with the 20-bit primitive index, as the
 * reference does (ORC_ERR_PANIC where its slice index would be out of bounds); lookup 1: the hit's
 * own object.  Per-BLAS arrays are concatenated: nodes at node_off[bl], triangles, normals (9 floats)
 * and texture coordinates (6 floats) at tri_off[bl] (tri_count[bl] of them), texels at byte
 * texel_off[bl] (tex_w[bl] x tex_h[bl] RGB8). */
int orc_render_scene(const float corners[9], const float view_inv[16], int width, int height, int accumulator,
                     const float* acc_params, int shader, const float* shader_params, const orc_tlas_node* tlas,
                     const uint32_t* blas_of, const float* xf, const float* inv, uint32_t nobj,
                     const orc_node* nodes, const uint32_t* node_off, const orc_tri* tris, const uint32_t* tri_off,
                     const uint32_t* tri_count, const float* normals, const float* tex_coords, const uint8_t* texels,
                     const uint64_t* texel_off, const uint32_t* tex_w, const uint32_t* tex_h, int lookup,
                     uint8_t* rgba, float* radiance);

/* --- bounce rays (not in the reference: cosine-weighted diffuse bounce) ---------------- */
int orc_bounce_ray(const orc_ray* primary, const orc_hit* hit, const orc_tri* tri, uint32_t seed,
                   uint32_t pixel, orc_ray* out);
int orc_bounce_rays(const orc_ray* primaries, const orc_hit* hits, uint32_t nrays, const orc_tri* tris,
                    uint32_t seed, orc_ray* out, uint8_t* valid);
/* Bounce rays of instanced hits (hit.inst selects the object, tri_off / blas_of as for the scene). */
int orc_scene_bounce_rays(const uint32_t* blas_of, const float* inv, const orc_tri* tris, const uint32_t* tri_off,
                          const orc_ray* primaries, const orc_hit* hits, uint32_t nrays, uint32_t seed, orc_ray* out,
                          uint8_t* valid);

#ifdef __cplusplus
}
#endif
#endif
