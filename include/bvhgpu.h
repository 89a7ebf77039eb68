/*
 * bvhgpu -- GB300 (sm_103a) ray-BVH hot path of lambdaxymox/bvhtracer behind a C ABI.
 *
 * The reference is a Rust crate with no FFI of its own; the entry points below are
 * what a Rust `extern "C"` block (bvhgpu-sys) binds to put the GPU path behind the
 * crate's own plug-in points.  Each declaration names the reference interface it
 * replaces (paths relative to the reference repository; BT = bvhtracer/).
 *
 * Conventions
 *  - Every function returns an int status (BVHGPU_OK == 0); no exception or abort
 *    crosses the ABI.  bvhgpu_last_error(ctx) gives a message for the last failure.
 *  - Plain C structs with fixed layouts (sizes asserted in the implementation).
 *  - Host pointers are caller-owned and only read/written during the call.  Device
 *    buffers behind BLAS / scene handles are owned by the context.
 *  - "_async" entry points take DEVICE pointers and a stream (NULL = the context's
 *    stream) and return before the work finishes; the others take HOST pointers and
 *    return after the results are in host memory.  Device ray arrays must be 16-byte
 *    aligned (a ray is read as two float4) and hit arrays 4-byte aligned, as memory from
 *    cudaMalloc / bvhgpu_device_alloc is; otherwise the call returns BVHGPU_ERR_INVALID_ARG.
 *  - A context is not thread-safe (one per host thread), like the reference's
 *    single-threaded Rc<RefCell<Model>> ownership (BT/src/model/model.rs:16-24).  Its
 *    launches share the context's work-queue counters and scratch, so work issued on
 *    different streams must not overlap on the GPU: use one stream per context (or order
 *    the streams with events); separate contexts run concurrently.
 *  - There is no CPU fallback: without a usable CUDA device bvhgpu_create fails.
 */
#ifndef BVHGPU_H
#define BVHGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes --------------------------------------------------------------- */
#define BVHGPU_OK 0
#define BVHGPU_ERR_INVALID_ARG 1   /* bad pointer, size, handle or malformed node array */
#define BVHGPU_ERR_OUT_OF_MEMORY 2
#define BVHGPU_ERR_CUDA 3          /* a CUDA runtime call failed */
#define BVHGPU_ERR_STACK_DEPTH 4   /* tree deeper than the traversal stack (device flag) */
#define BVHGPU_ERR_STEP_CAP 5      /* a traversal exceeded its step cap (corrupt tree) */
#define BVHGPU_ERR_BUILD 6         /* the reference's BvhBuilder would panic on this mesh */
#define BVHGPU_ERR_NO_DEVICE 7
#define BVHGPU_ERR_TOO_LARGE 8     /* input larger than a fixed-size entry point accepts */
#define BVHGPU_ERR_DEADLINE 9      /* a persistent launch ran past bvhgpu_set_deadline's budget */

/* ---- data layouts ------------------------------------------------------------------- */

/* BvhNode (BT/src/model/bvh.rs:129-134): 32 bytes, leaf iff primitive_count > 0; for a
 * branch left_first is the left child (right = left + 1, bvh.rs:111-113), for a leaf the
 * first primitive.  Node 0 is the root, node 1 an unused filler (bvh.rs:514-517). */
typedef struct bvhgpu_node {
    float bounds_min[3];
    float bounds_max[3];
    uint32_t primitive_count;
    uint32_t left_first;
} bvhgpu_node;

/* Triangle<f32> (BT/src/geometry/triangle.rs:11-17): three vertices, 36 bytes. */
typedef struct bvhgpu_triangle {
    float vertices[9];
} bvhgpu_triangle;

/* Ray<f32> (BT/src/query/ray.rs:9-35) without the derived reciprocal direction (the
 * kernels recompute 1/d with the same IEEE division).  t = FLT_MAX for Ray::from_origin_dir. */
typedef struct bvhgpu_ray {
    float origin[3];
    float t;
    float direction[3];
    uint32_t reserved;
} bvhgpu_ray;

/* Intersection (BT/src/query/intersection.rs:83-92) reduced to the hit record: t, u, v of
 * SurfaceInteraction and separate 32-bit primitive / instance ids (the reference packs
 * them in 20 + 12 bits, intersection.rs:41-66).  A miss (Option::None) is
 * t = FLT_MAX, u = v = 0, prim = inst = BVHGPU_MISS. */
typedef struct bvhgpu_hit {
    float t, u, v;
    uint32_t prim;
    uint32_t inst;
} bvhgpu_hit;
#define BVHGPU_MISS 0xFFFFFFFFu

/* TlasNode (BT/src/scene/tlas.rs:41-46): left_right packs two 16-bit node indices with the
 * reference's swapped getters (tlas.rs:17-32); leaf iff left_right == 0. */
typedef struct bvhgpu_tlas_node {
    float bounds_min[3];
    float bounds_max[3];
    uint32_t left_right;
    uint32_t blas;
} bvhgpu_tlas_node;

/* Camera::get_ray_world inputs (BT/src/camera/camera.rs:994-1010): the eye-space frustum
 * corners (top-left, top-right, bottom-left) and view_matrix_inv, column-major. */
typedef struct bvhgpu_camera {
    float top_left[3];
    float top_right[3];
    float bottom_left[3];
    float view_inv[16];
} bvhgpu_camera;

/* One scene of an uneven batch: rays [ray_offset, ray_offset + ray_count) of the batch's
 * ray array are traced against BLAS `blas`. */
typedef struct bvhgpu_batch_item {
    uint32_t blas;
    uint32_t ray_offset;
    uint32_t ray_count;
    uint32_t reserved;
} bvhgpu_batch_item;

/* Accumulators (BT/src/renderer.rs:108-110, 134-286) and pixel shaders (:112-222). */
#define BVHGPU_ACC_INTERSECTION 0  /* IntersectionAccumulator: params hit rgb, miss rgb */
#define BVHGPU_ACC_DEPTH 1         /* DepthAccumulator */
#define BVHGPU_ACC_UV 2            /* UvMappingAccumulator */
#define BVHGPU_ACC_NORMAL 3        /* NormalMappingAccumulator: params = object transform (16) */
#define BVHGPU_ACC_TEXTURE 4       /* TextureMaterialAccumulator: bvhgpu_render_textured only */
#define BVHGPU_SHADER_RADIANCE 0      /* RadianceToRgbShader */
#define BVHGPU_SHADER_INTERSECTION 1  /* IntersectionShader: params hit rgba, miss rgba */
#define BVHGPU_SHADER_DEPTH 2         /* DepthMappingShader: params scale, offset */

/* Trace modes for the bounce and batch entry points. */
#define BVHGPU_MODE_PLAIN 0       /* one launch per scene / pass */
#define BVHGPU_MODE_PERSISTENT 1  /* one persistent work-stealing launch */

typedef struct bvhgpu_ctx bvhgpu_ctx;
typedef void* bvhgpu_stream; /* a cudaStream_t */

/* ---- context ------------------------------------------------------------------------ */
/* Replaces nothing in the reference (it has no device); owns the stream and buffers. */
int bvhgpu_create(bvhgpu_ctx** out, int device);
int bvhgpu_destroy(bvhgpu_ctx* ctx);
const char* bvhgpu_last_error(const bvhgpu_ctx* ctx);
/* Number of kernels this library launched since load (all contexts). */
uint64_t bvhgpu_launch_count(void);
/* Waits for the context's stream and reports any device-side error flag. */
int bvhgpu_sync(bvhgpu_ctx* ctx);
bvhgpu_stream bvhgpu_get_stream(bvhgpu_ctx* ctx);
/* A time budget for each persistent launch of this context (the single-BLAS bounce, batch, scene
 * bounce and Lambertian forward launches), in nanoseconds of the device clock from the start of
 * each of its warps; 0 (the default) means none.  A launch past it stops taking and tracing rays
 * and the next synchronising call (or bvhgpu_sync) returns BVHGPU_ERR_DEADLINE; that launch's
 * outputs are then incomplete, and the context stays usable.  For a serving caller that must
 * bound a frame's time; no reference counterpart (the reference has no time limit).  Applies to
 * launches issued after the call; not allowed during graph capture. */
int bvhgpu_set_deadline(bvhgpu_ctx* ctx, uint64_t ns);

/* ---- memory helpers (for callers without their own CUDA allocator) ------------------- */
int bvhgpu_device_alloc(bvhgpu_ctx* ctx, size_t bytes, void** out);
int bvhgpu_device_free(bvhgpu_ctx* ctx, void* p);
int bvhgpu_host_alloc(bvhgpu_ctx* ctx, size_t bytes, void** out); /* pinned */
int bvhgpu_host_free(bvhgpu_ctx* ctx, void* p);
int bvhgpu_copy_to_device(bvhgpu_ctx* ctx, void* dst, const void* src, size_t bytes, bvhgpu_stream s);
int bvhgpu_copy_to_host(bvhgpu_ctx* ctx, void* dst, const void* src, size_t bytes, bvhgpu_stream s);
int bvhgpu_memset_device(bvhgpu_ctx* ctx, void* dst, int value, size_t bytes, bvhgpu_stream s);
/* Writes a buffer larger than L2 so the next launch starts with a cold cache. */
int bvhgpu_flush_l2(bvhgpu_ctx* ctx, bvhgpu_stream s);

/* ---- timing ---------------------------------------------------------------------------- */
int bvhgpu_event_create(bvhgpu_ctx* ctx, void** ev);
int bvhgpu_event_destroy(bvhgpu_ctx* ctx, void* ev);
int bvhgpu_event_record(bvhgpu_ctx* ctx, void* ev, bvhgpu_stream s);
int bvhgpu_event_elapsed_ms(bvhgpu_ctx* ctx, void* start, void* stop, float* ms);
/* Per-kernel timing: while enabled, every launch is bracketed by events on its own stream.
 * bvhgpu_profile_read waits and fills per-kernel total ms and launch counts (arrays of
 * BVHGPU_KERNEL_COUNT entries, indexed by the BVHGPU_K_* ids) and resets the table. */
#define BVHGPU_K_TRACE_BLAS 0
#define BVHGPU_K_TRACE_SCENE 1
#define BVHGPU_K_PERSISTENT_BOUNCE 2
#define BVHGPU_K_BOUNCE_GEN 3
#define BVHGPU_K_TRACE_QUEUE 4
#define BVHGPU_K_TRACE_BATCH 5
#define BVHGPU_K_REFIT 6
#define BVHGPU_K_TLAS_BUILD 7
#define BVHGPU_K_RENDER 8
#define BVHGPU_K_OTHER 9
#define BVHGPU_K_LAMBERT_FORWARD 10
#define BVHGPU_K_LAMBERT_ADJOINT 11
#define BVHGPU_K_SCENE_BOUNCE 12
#define BVHGPU_KERNEL_COUNT 13
int bvhgpu_profile_enable(bvhgpu_ctx* ctx, int enable);
int bvhgpu_profile_read(bvhgpu_ctx* ctx, double* ms, uint64_t* launches);

/* BvhBuilder::build_for on the GPU: the same nodes, triangle order and permutation as
 * bvhgpu_build_bvh_host / bvhgpu_build_bvh_host_indexed, bit for bit (BVHGPU_ERR_BUILD where the
 * reference panics).  mesh (host) is reordered in place; nodes_out holds 2n nodes; perm_out (n
 * entries, may be NULL) gets the input index of the triangle at each position.  Synchronous. */
int bvhgpu_build_bvh_device(bvhgpu_ctx* ctx, bvhgpu_triangle* mesh, uint32_t n, bvhgpu_node* nodes_out,
                            uint32_t* nodes_used, uint32_t* perm_out);
/* Build on the GPU and upload as a BLAS in one call; mesh (host) is reordered in place. */
int bvhgpu_blas_build(bvhgpu_ctx* ctx, bvhgpu_triangle* mesh, uint32_t n, uint32_t* blas_id);

/* ---- mesh decoders (host; no context needed) ------------------------------------------------ */
/* BVHGPU_MESH_TRI: the reference's `.tri` loader (BT/tri_loader/src/loader.rs, lexer.rs) and
 * TriMeshDecoder (BT/src/mesh/decoders.rs:108-133): nine floats per triangle, the face normal
 * normalize(normalize(v2-v0) x normalize(v1-v0)) at every corner, zero texture coordinates.
 * BVHGPU_MESH_OBJ: Wavefront `.obj`, first object only, with ObjMeshDecoder's per-corner normals
 * and texture coordinates (decoders.rs:157-215; f64 values cast to f32; polygons as fans).
 * Writes min(cap, n) triangles (36 B), normals (9 floats) and uvs (6 floats) where the pointers
 * are not NULL and *ntris = n; call with cap = 0 to size the buffers.  A decoding error returns
 * BVHGPU_ERR_INVALID_ARG with the line and reason in err (errlen bytes, may be NULL). */
#define BVHGPU_MESH_TRI 0
#define BVHGPU_MESH_OBJ 1
int bvhgpu_mesh_decode(const char* text, size_t len, int format, bvhgpu_triangle* tris, float* normals, float* uvs,
                       uint32_t cap, uint32_t* ntris, char* err, size_t errlen);
int bvhgpu_mesh_decode_file(const char* path, int format, bvhgpu_triangle* tris, float* normals, float* uvs,
                            uint32_t cap, uint32_t* ntris, char* err, size_t errlen);

/* ---- triangle list, no BVH ----------------------------------------------------------------- */
/* Triangle::intersect / Triangle::intersect_mut (BT/src/geometry/triangle.rs:42-108) of every
 * ray against every triangle of a list, in index order (brute force, tiled through shared memory).
 *  BVHGPU_LIST_CLOSEST: Triangle::intersect with a BVH leaf's strict `<`: the first triangle with
 *                       the smallest t; a miss is the sentinel.
 *  BVHGPU_LIST_MUT:     Triangle::intersect_mut applied in order to one Intersection per ray:
 *                       every triangle that reports a hit sets t = min(t, its t) and overwrites
 *                       u and v (also when its t is larger); prim = the last such triangle.
 * Hit records carry inst = 0 for a hit. */
#define BVHGPU_LIST_CLOSEST 0
#define BVHGPU_LIST_MUT 1
int bvhgpu_triangles_intersect(bvhgpu_ctx* ctx, const bvhgpu_triangle* tris, uint32_t ntris, const bvhgpu_ray* rays,
                               uint32_t n, int mode, bvhgpu_hit* hits);
int bvhgpu_triangles_intersect_async(bvhgpu_ctx* ctx, const bvhgpu_triangle* d_tris, uint32_t ntris,
                                     const bvhgpu_ray* d_rays, uint32_t n, int mode, bvhgpu_hit* d_hits,
                                     bvhgpu_stream s);

/* ---- BLAS -------------------------------------------------------------------------------- */
/* BvhBuilder::build_for (BT/src/model/bvh.rs:524-541) on the host: the reference's SAH binned
 * build (8 bins), reordering `mesh` in place.  nodes_out must hold 2*n nodes. */
int bvhgpu_build_bvh_host(bvhgpu_triangle* mesh, uint32_t n, bvhgpu_node* nodes_out, uint32_t* nodes_used);

/* Same build, also writing perm_out[i] = the input index of the triangle that ends at position i
 * (n entries), so that an indexed mesh's faces can follow the reordering. */
int bvhgpu_build_bvh_host_indexed(bvhgpu_triangle* mesh, uint32_t n, bvhgpu_node* nodes_out, uint32_t* nodes_used,
                                  uint32_t* perm_out);

/* Upload a reference-built BVH as-is (the node array of Bvh, bvh.rs:227-233, and the mesh's
 * primitives, BT/src/mesh/mesh.rs:126-134).  Validates the tree; the handle replaces
 * ModelInstance's Bvh + mesh pair (BT/src/model/model.rs:16-33). */
int bvhgpu_blas_upload(bvhgpu_ctx* ctx, const bvhgpu_node* nodes, uint32_t nodes_used,
                       const bvhgpu_triangle* tris, uint32_t ntris, uint32_t* blas_id);
int bvhgpu_blas_free(bvhgpu_ctx* ctx, uint32_t blas_id);
int bvhgpu_blas_info(bvhgpu_ctx* ctx, uint32_t blas_id, uint32_t* nodes_used, uint32_t* ntris, uint32_t* depth);
/* Size of the hidden trees the library keeps under the BLAS's large leaves (leaves of at least 16
 * triangles): nodes, triangle pairs and the deepest tree's depth below its leaf.  A hidden box is
 * skipped for a ray only when provably no triangle in it is accepted at or below the ray's closest
 * t, and ties keep the lowest triangle index, so results equal the reference's in-order leaf loop
 * (bvh.rs:250-258).  Hidden interior nodes have 2 to 4 children.  No reference counterpart:
 * exposed for tests and tuning.  Any pointer may be NULL. */
int bvhgpu_blas_hidden(bvhgpu_ctx* ctx, uint32_t blas_id, uint32_t* nodes, uint32_t* pairs, uint32_t* depth);
/* The hidden trees' device data, for tests (no reference counterpart): `nodes` gets the hidden node
 * records (bvhgpu_blas_hidden's node count x 8 floats: lo.xyz, first, hi.xyz, count, the integers
 * as their bits), `cones` the cone records (*ncones x 8 floats: axis.xyz, cos_phi, sin_phi, nmin,
 * Q, B), `slots` the two triangle indices of each hidden pair (pairs x 2, 0xFFFFFFFF for a padding
 * slot) and `table` the per-triangle entries ((ntris + 1) & ~1 entries x 2: {first, count} of the
 * hidden root at a large leaf's first triangle, else {0, 0}).  Any array may be NULL; *ncones
 * (if not NULL) gets the number of cone records.  Synchronous. */
int bvhgpu_blas_hidden_download(bvhgpu_ctx* ctx, uint32_t blas_id, float* nodes, float* cones, uint32_t* slots,
                                uint32_t* table, uint32_t* ncones);
/* bvhgpu_blas_intersect_async's traversal with work counters (device buffers; synchronous): the
 * hits (identical to the plain call's) and, summed over the rays, counts[0..6] = reference
 * interior nodes visited, hidden child boxes tested, hidden trees entered, hidden triangle
 * pairs tested, triangles tested lane by lane, triangles tested by the warp, cone records read
 * on entering another cone's subtree -- the node and triangle bytes each ray fetched.  No
 * reference counterpart: for measurement. */
int bvhgpu_blas_trace_counts(bvhgpu_ctx* ctx, uint32_t blas_id, const bvhgpu_ray* d_rays, uint32_t n,
                             bvhgpu_hit* d_hits, uint64_t counts[7]);
/* New vertex positions (same triangle order), e.g. an animated mesh before refit. */
int bvhgpu_blas_update_vertices(bvhgpu_ctx* ctx, uint32_t blas_id, const bvhgpu_triangle* tris);
int bvhgpu_blas_update_vertices_async(bvhgpu_ctx* ctx, uint32_t blas_id, const bvhgpu_triangle* d_tris,
                                      bvhgpu_stream s);
/* Bvh::refit (bvh.rs:469-493) / ModelInstance::refit (model.rs:31-33) on the GPU. */
int bvhgpu_blas_refit(bvhgpu_ctx* ctx, uint32_t blas_id);
int bvhgpu_blas_refit_async(bvhgpu_ctx* ctx, uint32_t blas_id, bvhgpu_stream s);
/* Read the node array back in the reference layout (nodes_used entries). */
int bvhgpu_blas_download_nodes(bvhgpu_ctx* ctx, uint32_t blas_id, bvhgpu_node* nodes);
/* Bvh::intersect (bvh.rs:307-309) / ModelInstance::intersect (model.rs:27-29) for a batch. */
int bvhgpu_blas_intersect(bvhgpu_ctx* ctx, uint32_t blas_id, const bvhgpu_ray* rays, uint32_t n,
                          bvhgpu_hit* hits);
int bvhgpu_blas_intersect_async(bvhgpu_ctx* ctx, uint32_t blas_id, const bvhgpu_ray* d_rays, uint32_t n,
                                bvhgpu_hit* d_hits, bvhgpu_stream s);

/* Primary rays + one cosine-weighted diffuse bounce per hit (not in the reference; the frame
 * pattern of its demos).  hits0[i] is ray i's closest hit, hits1[i] the hit of its bounce
 * (miss when ray i missed).  mode: BVHGPU_MODE_PLAIN (trace, compact, trace) or
 * BVHGPU_MODE_PERSISTENT (one work-stealing launch).  n_bounce (may be NULL) receives the
 * number of bounce rays traced.  The launch reads the rays and writes the hits in place when the
 * buffers are page-locked (bvhgpu_host_alloc), or ordinary host memory on a device that accesses
 * it coherently (Grace-attached GPUs; the hit arrays' pages are written once by the CPU first);
 * otherwise they are staged through the context's device buffers. */
int bvhgpu_blas_trace_bounce(bvhgpu_ctx* ctx, uint32_t blas_id, const bvhgpu_ray* rays, uint32_t n,
                             uint32_t seed, int mode, bvhgpu_hit* hits0, bvhgpu_hit* hits1, uint32_t* n_bounce);
int bvhgpu_blas_trace_bounce_async(bvhgpu_ctx* ctx, uint32_t blas_id, const bvhgpu_ray* d_rays, uint32_t n,
                                   uint32_t seed, int mode, bvhgpu_hit* d_hits0, bvhgpu_hit* d_hits1,
                                   bvhgpu_stream s);
/* The bounce rays the plain mode traced, in pixel order (valid[i] = 0 where none). */
int bvhgpu_blas_bounce_rays(bvhgpu_ctx* ctx, uint32_t blas_id, const bvhgpu_ray* rays, uint32_t n,
                            uint32_t seed, bvhgpu_ray* out, uint8_t* valid);

/* Uneven batch of scenes in one call: Scene::intersect repeated over many scenes.
 * mode BVHGPU_MODE_PLAIN launches once per item; BVHGPU_MODE_PERSISTENT runs one
 * work-stealing launch over all items, from a device table of the items that the context keeps
 * and rebuilds (synchronously) when the item list changes -- so under graph capture
 * (bvhgpu_graph_begin) a persistent batch must use the item list of an earlier call, else
 * BVHGPU_ERR_INVALID_ARG. */
int bvhgpu_trace_batch(bvhgpu_ctx* ctx, const bvhgpu_batch_item* items, uint32_t nitems,
                       const bvhgpu_ray* rays, uint32_t nrays, int mode, bvhgpu_hit* hits);
int bvhgpu_trace_batch_async(bvhgpu_ctx* ctx, const bvhgpu_batch_item* items, uint32_t nitems,
                             const bvhgpu_ray* d_rays, uint32_t nrays, int mode, bvhgpu_hit* d_hits,
                             bvhgpu_stream s);

/* ---- scene / TLAS ----------------------------------------------------------------------- */
/* SceneBuilder::build (BT/src/scene/scene.rs:224-234): objects i = 0..n-1 instance BLAS
 * blas_ids[i].  Transforms start as identity.  At most 32,768 objects: the TLAS's 2n nodes are
 * addressed by LeftRightIndex's 16-bit halves (tlas.rs:18-22). */
int bvhgpu_scene_create(bvhgpu_ctx* ctx, const uint32_t* blas_ids, uint32_t nobjects, uint32_t* scene_id);
int bvhgpu_scene_free(bvhgpu_ctx* ctx, uint32_t scene_id);
/* SceneObject::set_transform (BT/src/scene/scene_object.rs:60-75) for all objects: the
 * transform and its cached inverse (TransformComponent3, BT/src/transform_component.rs:24-27),
 * 16 floats each, column-major.  World bounds are recomputed on the GPU at rebuild. */
int bvhgpu_scene_set_transforms(bvhgpu_ctx* ctx, uint32_t scene_id, const float* xf, const float* inv);
int bvhgpu_scene_set_transforms_async(bvhgpu_ctx* ctx, uint32_t scene_id, const float* d_xf,
                                      const float* d_inv, bvhgpu_stream s);
/* Scene::rebuild / Tlas::rebuild (scene.rs:36-38, tlas.rs:204-250) on the GPU. */
int bvhgpu_scene_rebuild(bvhgpu_ctx* ctx, uint32_t scene_id);
int bvhgpu_scene_rebuild_async(bvhgpu_ctx* ctx, uint32_t scene_id, bvhgpu_stream s);
int bvhgpu_scene_download_tlas(bvhgpu_ctx* ctx, uint32_t scene_id, bvhgpu_tlas_node* nodes, uint32_t* nodes_used);
/* Scene::intersect (scene.rs:32-34, tlas.rs:123-177, scene_object.rs:78-89).  Unlike the
 * reference (which always reports instance 0) hit.inst is the object index. */
int bvhgpu_scene_intersect(bvhgpu_ctx* ctx, uint32_t scene_id, const bvhgpu_ray* rays, uint32_t n,
                           bvhgpu_hit* hits);
int bvhgpu_scene_intersect_async(bvhgpu_ctx* ctx, uint32_t scene_id, const bvhgpu_ray* d_rays, uint32_t n,
                                 bvhgpu_hit* d_hits, bvhgpu_stream s);

/* Primary rays + one cosine-weighted bounce per hit over a scene (the instanced frame), one
 * persistent launch; as bvhgpu_blas_trace_bounce_async but two-level, hits carry the instance. */
int bvhgpu_scene_trace_bounce_async(bvhgpu_ctx* ctx, uint32_t scene_id, const bvhgpu_ray* d_rays, uint32_t n,
                                    uint32_t seed, bvhgpu_hit* d_hits0, bvhgpu_hit* d_hits1, bvhgpu_stream s);
/* The bounce rays of a scene frame in pixel order (host in/out; valid[i] = 0 where none). */
int bvhgpu_scene_bounce_rays(bvhgpu_ctx* ctx, uint32_t scene_id, const bvhgpu_ray* rays, uint32_t n, uint32_t seed,
                             bvhgpu_ray* out, uint8_t* valid);
/* Current object transforms and cached inverses (16 floats each, column-major). */
int bvhgpu_scene_download_transforms(bvhgpu_ctx* ctx, uint32_t scene_id, float* xf, float* inv);

/* ---- animated frames in a CUDA graph (the per-frame pattern of the reference's demos) ------------ */
/* Closed-form animation driven by a time value in device memory (so that a captured graph replays
 * with the current time): radial vertex wobble v = dir * (r0 + amp * sin(freq * t + phase)) of a
 * mesh (then bvhgpu_mesh_update_async regenerates and refits its BLAS), and per-instance rotation
 * R_i(t) = R0_i * Rot(axis_i, omega_i * t) with uniform scale and translation, written as the
 * scene's transforms and inverses (then bvhgpu_scene_rebuild_async). */
int bvhgpu_mesh_wobble_async(bvhgpu_ctx* ctx, uint32_t mesh_id, const float* d_dirs, const float* d_r0,
                             const float* d_phase, float amp, float freq, const float* d_time, bvhgpu_stream s);
int bvhgpu_scene_animate_async(bvhgpu_ctx* ctx, uint32_t scene_id, const float* d_rot0, const float* d_axis,
                               const float* d_omega, const float* d_scale, const float* d_trans, const float* d_time,
                               bvhgpu_stream s);
int bvhgpu_advance_time_async(bvhgpu_ctx* ctx, float* d_time, float dt, bvhgpu_stream s);
/* Stream capture of the context's stream: every _async call with a NULL stream between begin and
 * end is recorded (no work runs), end instantiates the graph; launch replays it. */
int bvhgpu_graph_begin(bvhgpu_ctx* ctx);
int bvhgpu_graph_end(bvhgpu_ctx* ctx, uint32_t* graph_id);
int bvhgpu_graph_launch(bvhgpu_ctx* ctx, uint32_t graph_id);
int bvhgpu_graph_free(bvhgpu_ctx* ctx, uint32_t graph_id);

/* ---- tiled render ----------------------------------------------------------------------- */
/* Integrator::evaluate for PathTracer (BT/src/renderer.rs:104-106, 345-384) on one BLAS:
 * 8x8 tiles, one ray per pixel through the pixel's top-left corner, accumulator + shader ->
 * RGBA8 (row-major, w*h*4 bytes, not flipped).  normals (9 floats per triangle, in the BLAS's
 * triangle order) only for BVHGPU_ACC_NORMAL.  Returns rays traced in *rays_traced. */
int bvhgpu_render(bvhgpu_ctx* ctx, uint32_t blas_id, const bvhgpu_camera* camera, int width, int height,
                  int accumulator, const float* acc_params, int shader, const float* shader_params,
                  const float* normals, uint8_t* rgba, uint64_t* rays_traced);
/* TextureMaterialAccumulator (BT/src/renderer.rs:289-334) + shader: the hit's texture coordinate
 * (per-corner tex_coords, 6 floats per triangle in the BLAS's triangle order, interpolated with the
 * barycentrics) looks up an RGB8 texture (texels, tex_w x tex_h, row-major) as
 * TextureMaterial::evaluate does (BT/src/materials/material.rs:44-52: (u * w) as usize % w). */
int bvhgpu_render_textured(bvhgpu_ctx* ctx, uint32_t blas_id, const bvhgpu_camera* camera, int width, int height,
                           const float* tex_coords, const uint8_t* texels, uint32_t tex_w, uint32_t tex_h,
                           int shader, const float* shader_params, uint8_t* rgba, uint64_t* rays_traced);

/* Shading data of a BLAS's model -- what Model holds beside the BVH (BT/src/model/model.rs:16-24,
 * mesh normals and texture coordinates of BT/src/mesh/mesh.rs, the texture of
 * BT/src/materials/material.rs) and what bvhgpu_render_scene's normal and texture accumulators read:
 * corner normals (9 floats per triangle), corner texture coordinates (6 floats per triangle), both
 * in the BLAS's triangle order, and an RGB8 texture (texels, tex_w x tex_h, row-major).  Each
 * pointer may be NULL (that array is kept as it is).  Synchronous (copies the data to the device). */
int bvhgpu_blas_set_shading(bvhgpu_ctx* ctx, uint32_t blas_id, const float* normals, const float* tex_coords,
                            const uint8_t* texels, uint32_t tex_w, uint32_t tex_h);
/* Integrator::evaluate for PathTracer on a whole Scene (BT/src/renderer.rs:104-106, 345-384 ->
 * Scene::intersect, BT/src/scene/scene.rs:32-34): every pixel's camera ray through the TLAS and the
 * instances' BLASes, then the accumulator (any BVHGPU_ACC_*) and the shader -> RGBA8 (row-major,
 * w*h*4 bytes).  acc_params only for BVHGPU_ACC_INTERSECTION (hit rgb, miss rgb); the normal
 * accumulator's transform is the looked-up object's own (SceneObject::get_transform).  The normal
 * and texture accumulators look up the model named by the hit's InstancePrimitiveIndex
 * (renderer.rs:258-263, 312-317):
 *  BVHGPU_LOOKUP_REFERENCE: what the reference computes -- its Bvh::intersect always packs
 *    instance 0 (bvh.rs:296, intersection.rs:63-66), so object 0's model and transform, with the
 *    primitive id's low 20 bits;
 *  BVHGPU_LOOKUP_HIT_OBJECT: the hit's own object and primitive.
 * A primitive outside the looked-up model's shading data (the reference panics: slice index out of
 * bounds), or a model without the needed data, returns BVHGPU_ERR_INVALID_ARG after the frame
 * (those pixels get zero radiance).  Returns rays traced in *rays_traced. */
#define BVHGPU_LOOKUP_REFERENCE 0
#define BVHGPU_LOOKUP_HIT_OBJECT 1
int bvhgpu_render_scene(bvhgpu_ctx* ctx, uint32_t scene_id, const bvhgpu_camera* camera, int width, int height,
                        int accumulator, const float* acc_params, int shader, const float* shader_params, int lookup,
                        uint8_t* rgba, uint64_t* rays_traced);

/* ---- differentiable Lambertian render (not in the reference) ----------------------------------- */
/* Indexed mesh over a BLAS: triangle i of the BLAS is (verts[faces[3i]], verts[faces[3i+1]],
 * verts[faces[3i+2]]), i.e. faces are given in the BLAS's triangle order (see
 * bvhgpu_build_bvh_host_indexed).  vnormals are per-vertex shading normals, interpolated with the
 * hit's barycentrics like NormalMappingAccumulator (BT/src/renderer.rs:268-272) and held fixed. */
int bvhgpu_mesh_create(bvhgpu_ctx* ctx, uint32_t blas_id, const uint32_t* faces, uint32_t nfaces, const float* verts,
                       const float* vnormals, uint32_t nverts, uint32_t* mesh_id);
int bvhgpu_mesh_free(bvhgpu_ctx* ctx, uint32_t mesh_id);
/* Device pointer of the mesh's vertex array (3 floats per vertex), e.g. for a custom update. */
int bvhgpu_mesh_vertices(bvhgpu_ctx* ctx, uint32_t mesh_id, float** d_verts);
/* New vertex positions from the host; the BLAS triangles are regenerated and refit. */
int bvhgpu_mesh_set_vertices(bvhgpu_ctx* ctx, uint32_t mesh_id, const float* verts);
/* Regenerate the BLAS triangles from the mesh's device vertices and refit (Bvh::refit). */
int bvhgpu_mesh_update_async(bvhgpu_ctx* ctx, uint32_t mesh_id, bvhgpu_stream s);
/* Forward: closest hit per ray, hit records {t, u, v, prim} written to d_hits (the checkpoint the
 * adjoint reuses), image[i] = max(0, n_hat . l_hat) with n the barycentric vertex normal and l the
 * direction from the hit point to the point light `light` (0 for a miss).  One persistent launch
 * under the BVHGPU_K_TRACE_BLAS launch config (shape, stack, leaf policy, refill).  Each pass
 * records which rays took long to trace, and the mesh's next pass starts those first, spread over
 * the launch (results never depend on it); the record takes 16 bytes per ray, allocated by the first
 * pass at a larger ray count (outside stream capture; a captured pass that finds it too small runs
 * without it).  Passes of one mesh must not run concurrently. */
int bvhgpu_lambert_forward_async(bvhgpu_ctx* ctx, uint32_t mesh_id, const bvhgpu_ray* d_rays, uint32_t n,
                                 const float light[3], float* d_image, bvhgpu_hit* d_hits, bvhgpu_stream s);
/* Mean squared error between image and target (n floats each, device), computed on the device in
 * double precision; waits for the stream. */
int bvhgpu_mse_loss(bvhgpu_ctx* ctx, const float* d_image, const float* d_target, uint32_t n, double* loss);
/* Adjoint of forward + mean squared error: adds dLoss/dvertex (3 floats per vertex) into d_grad,
 * from the checkpointed hit records (no re-trace; visibility held fixed). */
int bvhgpu_lambert_adjoint_async(bvhgpu_ctx* ctx, uint32_t mesh_id, const bvhgpu_ray* d_rays, uint32_t n,
                                 const float light[3], const bvhgpu_hit* d_hits, const float* d_image,
                                 const float* d_target, float* d_grad, bvhgpu_stream s);
/* Gradient-descent step on the mesh vertices: verts -= lr * grad, then grad = 0 (call
 * bvhgpu_mesh_update_async before the next forward). */
int bvhgpu_mesh_sgd_step_async(bvhgpu_ctx* ctx, uint32_t mesh_id, float* d_grad, float lr, bvhgpu_stream s);

/* ---- launch configuration and autotuning (not in the reference) ------------------------------ */
/* The traversal kernels BVHGPU_K_TRACE_BLAS (also the bounce pass of BVHGPU_MODE_PLAIN and the
 * per-scene launches of a plain batch), BVHGPU_K_TRACE_SCENE, BVHGPU_K_PERSISTENT_BOUNCE,
 * BVHGPU_K_TRACE_BATCH and BVHGPU_K_SCENE_BOUNCE are compiled in several variants, and a context
 * holds one config per kernel.  Every config gives bit-identical results; it only changes speed. */
#define BVHGPU_BIG_LEAF_NEVER 0xFFFFFFFFu
typedef struct bvhgpu_tune_config {
    /* launch shape: threads per block and the blocks per SM that __launch_bounds__ sizes the
     * register budget for (65536 / (block * min_blocks) registers per thread).  Compiled shapes:
     * (128, 1), (128, 5), (128, 6), (128, 8), (64, 1). */
    uint32_t block;
    uint32_t min_blocks;
    /* traversal stack entries per ray: 8 or 32 (the newest 4 in registers, the rest in shared
     * memory) or 256 (local memory).  0, or fewer than the tree needs: the smallest that holds it. */
    uint32_t stack;
    /* leaf layout: a leaf with more triangles than this is tested by the whole warp on the paired
     * f32x2 triangle layout, smaller ones by their own lane on the float4 layout;
     * BVHGPU_BIG_LEAF_NEVER = every leaf by its lane. */
    uint32_t big_leaf;
    /* ray batch of the persistent kernels: a warp fetches new rays once this many of its lanes
     * are idle (1..32; a warp whose lanes are all idle always fetches). */
    uint32_t refill;
    /* hidden trees: a ray walks a large leaf's hidden tree (bvhgpu_blas_hidden) when its cull
     * margin there, in thousandths of a triangle's barycentric range, is below this; otherwise the
     * leaf is tested in order (big_leaf decides by whom).  0 = never. */
    uint32_t hidden;
} bvhgpu_tune_config;
/* Defaults (the tuner's picks on GB300): block 128, min_blocks 5, stack 256, big_leaf 16, refill 8,
 * hidden 2000; for the single-ray kernels (TRACE_BLAS, TRACE_SCENE) refill 1. */
int bvhgpu_tune_get(bvhgpu_ctx* ctx, int kernel, bvhgpu_tune_config* out);
/* BVHGPU_ERR_INVALID_ARG for a kernel that is not tunable or a shape / stack not compiled. */
int bvhgpu_tune_set(bvhgpu_ctx* ctx, int kernel, const bvhgpu_tune_config* cfg);
/* The candidate values the tuner searches, as a list of configs (cap entries at most; *count
 * gets the full number): every compiled shape x stack, big_leaf in {8, 16, 32, 64, NEVER},
 * refill in {1, 8, 16} (refill only for the persistent kernels) and hidden in
 * {0, 100, 250, 500, 1000}. */
int bvhgpu_tune_space(int kernel, bvhgpu_tune_config* out, uint32_t cap, uint32_t* count);

/* One call for the tuner to time: the fields a kernel needs, others 0 / NULL.
 *   TRACE_BLAS:        target = BLAS id, d_rays, n, d_hits0 (bvhgpu_blas_intersect_async); or,
 *                      with nitems > 0, the plain batch of `items` (one launch per item)
 *   PERSISTENT_BOUNCE: target = BLAS id, d_rays, n, seed, d_hits0, d_hits1
 *   TRACE_SCENE:       target = scene id, d_rays, n, d_hits0
 *   SCENE_BOUNCE:      target = scene id, d_rays, n, seed, d_hits0, d_hits1
 *   TRACE_BATCH:       items, nitems, d_rays, n (= total rays), d_hits0 */
typedef struct bvhgpu_tune_job {
    int kernel;
    uint32_t target;
    const bvhgpu_ray* d_rays;
    uint32_t n;
    uint32_t seed;
    bvhgpu_hit* d_hits0;
    bvhgpu_hit* d_hits1;
    const bvhgpu_batch_item* items;
    uint32_t nitems;
} bvhgpu_tune_job;
/* Times the job under candidate configs -- a coordinate search from the current config over
 * launch shape, stack, big_leaf, refill and hidden, two sweeps; each candidate runs once untimed, then
 * `reps` times bracketed by events on the context's stream (median kept) -- stores the fastest
 * in the context and returns it with its ms per call (either pointer may be NULL).  The job's
 * outputs are overwritten.  Synchronous; not allowed during graph capture. */
int bvhgpu_autotune(bvhgpu_ctx* ctx, const bvhgpu_tune_job* job, uint32_t reps, bvhgpu_tune_config* best,
                    float* best_ms);

/* ---- rigid-body physics driving instance transforms (BT/src/physics/, scene.rs:40-50) ---------- */
/* RigidBody (physics/rigid_body.rs:74-122) as a plain struct; matrices column-major [col][row]. */
typedef struct bvhgpu_rigid_body {
    float inverse_mass;
    float inverse_inertia[9];        /* body space */
    float linear_drag, angular_drag;
    float position[3];
    float orientation[4];            /* quaternion s, x, y, z */
    float velocity[3];
    float rotation[3];               /* angular velocity */
    float inverse_inertia_world[9];
    float motion;
    uint32_t is_awake, can_sleep;
    float transform[16];             /* body space to world space */
    float force_accum[3], torque_accum[3];
    float acceleration[3], last_frame_acceleration[3];
} bvhgpu_rigid_body;
/* ForceGenerator (physics/force_generator.rs): Gravity (gravity), or Spring from `body`'s
 * spring_point to `other`'s other_point (body-space points) with spring_constant, rest_length. */
#define BVHGPU_FORCE_GRAVITY 0
#define BVHGPU_FORCE_SPRING 1
typedef struct bvhgpu_force_generator {
    uint32_t kind, body, other, reserved;
    float gravity[3];
    float spring_point[3];
    float other_point[3];
    float spring_constant, rest_length;
} bvhgpu_force_generator;
/* World (physics/world.rs): bodies and the force registry, in registration order. */
int bvhgpu_world_create(bvhgpu_ctx* ctx, const bvhgpu_rigid_body* bodies, uint32_t nbodies,
                        const bvhgpu_force_generator* gens, uint32_t ngens, uint32_t* world_id);
int bvhgpu_world_free(bvhgpu_ctx* ctx, uint32_t world_id);
/* World::start_frame: clear the accumulators and RigidBody::calculate_derived_data. */
int bvhgpu_world_start_frame_async(bvhgpu_ctx* ctx, uint32_t world_id, bvhgpu_stream s);
/* World::run_physics(dt): the registry's forces, then RigidBody::integrate (Newton-Euler). */
int bvhgpu_world_step_async(bvhgpu_ctx* ctx, uint32_t world_id, float dt, bvhgpu_stream s);
int bvhgpu_world_download(bvhgpu_ctx* ctx, uint32_t world_id, bvhgpu_rigid_body* bodies_out);
/* Binds scene objects to bodies: object i follows body body_of[i] (0xFFFFFFFF: none) with its
 * initial transform transform_init[16 i..] (SceneObjectBuilder::with_transform). */
int bvhgpu_scene_bind_world(bvhgpu_ctx* ctx, uint32_t scene_id, uint32_t world_id, const uint32_t* body_of,
                            const float* transform_init);
/* Scene::run(dt) (scene.rs:40-50): World::run_physics, SceneObject::update_transform of every bound
 * object (body transform * initial transform, and its inverse), Scene::rebuild.  Capturable. */
int bvhgpu_scene_run_async(bvhgpu_ctx* ctx, uint32_t scene_id, float dt, bvhgpu_stream s);

/* ---- refit without allocation ----------------------------------------------------------------- */
/* No counterpart in the reference.  For callers that cannot call cudaMalloc: engines that own all
 * device memory through a pool reserved at start-up, or latency-critical threads on which a driver
 * allocation (which can synchronise the device) is not allowed.  Refits, in place, a node array the
 * caller owns on the device (reference layout, nodes_used entries) against the caller's device
 * triangles (ntris x 36 bytes), with the same results as bvhgpu_blas_refit.  Allocates nothing and
 * needs no context: its scratch is a fixed device array of 8 MiB that every GPU which loads the
 * library holds until the process exits, so nodes_used may be at most BVHGPU_NOALLOC_MAX_NODES
 * (larger arrays return BVHGPU_ERR_TOO_LARGE).  Runs asynchronously on `stream` (NULL = legacy
 * default stream) on the current device.  The first call on a device looks up the scratch array's
 * device address (cudaGetSymbolAddress) with that device current; make that first call before any
 * stream capture.  Every call shares the one scratch array and resets the part it uses, so calls
 * whose work overlaps on the GPU (different streams, or different threads with the same device)
 * race and must be serialised by the caller.  A process that calls cudaDeviceReset on a device must
 * not call this entry point on that device afterwards (the looked-up address belonged to the
 * destroyed context).  If d_status (device, caller-owned, may be NULL) is given, the value 1 is
 * OR-ed in for a branch whose child index is out of range or not above its own, 2 for a leaf
 * addressing triangles past ntris, 4 for a node that two branches claim as a child; such nodes
 * are skipped, and their ancestors keep their old bounds.  The caller clears it. */
#define BVHGPU_NOALLOC_MAX_NODES (1u << 20)
int bvhgpu_refit_noalloc(bvhgpu_node* d_nodes, uint32_t nodes_used, const bvhgpu_triangle* d_tris, uint32_t ntris,
                         bvhgpu_stream stream, uint32_t* d_status);

#ifdef __cplusplus
}
#endif
#endif /* BVHGPU_H */
