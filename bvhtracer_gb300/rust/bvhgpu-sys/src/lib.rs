//! Raw bindings of the bvhgpu C ABI (include/bvhgpu.h), generated by gen_bindings.py -- do not
//! edit by hand.  Every function returns a status (BVHGPU_OK = 0); see the header for each
//! entry point's contract and the reference interface it replaces.
#![allow(non_camel_case_types)]
#![no_std]

pub use core::ffi::{c_char, c_int, c_void};

/// Opaque library context (one per host thread).
#[repr(C)]
pub struct bvhgpu_ctx {
    _private: [u8; 0],
}
/// A cudaStream_t; null selects the context's own stream.
pub type bvhgpu_stream = *mut c_void;

pub const BVHGPU_OK: c_int = 0;
pub const BVHGPU_ERR_INVALID_ARG: c_int = 1;
pub const BVHGPU_ERR_OUT_OF_MEMORY: c_int = 2;
pub const BVHGPU_ERR_CUDA: c_int = 3;
pub const BVHGPU_ERR_STACK_DEPTH: c_int = 4;
pub const BVHGPU_ERR_STEP_CAP: c_int = 5;
pub const BVHGPU_ERR_BUILD: c_int = 6;
pub const BVHGPU_ERR_NO_DEVICE: c_int = 7;
pub const BVHGPU_ERR_TOO_LARGE: c_int = 8;
pub const BVHGPU_ERR_DEADLINE: c_int = 9;
pub const BVHGPU_MISS: u32 = 0xFFFF_FFFF;
pub const BVHGPU_ACC_INTERSECTION: c_int = 0;
pub const BVHGPU_ACC_DEPTH: c_int = 1;
pub const BVHGPU_ACC_UV: c_int = 2;
pub const BVHGPU_ACC_NORMAL: c_int = 3;
pub const BVHGPU_ACC_TEXTURE: c_int = 4;
pub const BVHGPU_SHADER_RADIANCE: c_int = 0;
pub const BVHGPU_SHADER_INTERSECTION: c_int = 1;
pub const BVHGPU_SHADER_DEPTH: c_int = 2;
pub const BVHGPU_MODE_PLAIN: c_int = 0;
pub const BVHGPU_MODE_PERSISTENT: c_int = 1;
pub const BVHGPU_K_TRACE_BLAS: c_int = 0;
pub const BVHGPU_K_TRACE_SCENE: c_int = 1;
pub const BVHGPU_K_PERSISTENT_BOUNCE: c_int = 2;
pub const BVHGPU_K_BOUNCE_GEN: c_int = 3;
pub const BVHGPU_K_TRACE_QUEUE: c_int = 4;
pub const BVHGPU_K_TRACE_BATCH: c_int = 5;
pub const BVHGPU_K_REFIT: c_int = 6;
pub const BVHGPU_K_TLAS_BUILD: c_int = 7;
pub const BVHGPU_K_RENDER: c_int = 8;
pub const BVHGPU_K_OTHER: c_int = 9;
pub const BVHGPU_K_LAMBERT_FORWARD: c_int = 10;
pub const BVHGPU_K_LAMBERT_ADJOINT: c_int = 11;
pub const BVHGPU_K_SCENE_BOUNCE: c_int = 12;
pub const BVHGPU_KERNEL_COUNT: c_int = 13;
pub const BVHGPU_MESH_TRI: c_int = 0;
pub const BVHGPU_MESH_OBJ: c_int = 1;
pub const BVHGPU_LIST_CLOSEST: c_int = 0;
pub const BVHGPU_LIST_MUT: c_int = 1;
pub const BVHGPU_LOOKUP_REFERENCE: c_int = 0;
pub const BVHGPU_LOOKUP_HIT_OBJECT: c_int = 1;
pub const BVHGPU_BIG_LEAF_NEVER: u32 = 0xFFFF_FFFF;
pub const BVHGPU_FORCE_GRAVITY: c_int = 0;
pub const BVHGPU_FORCE_SPRING: c_int = 1;
pub const BVHGPU_NOALLOC_MAX_NODES: u32 = 1 << 20;

#[repr(C)]
#[derive(Copy, Clone, Debug, Default)]
pub struct bvhgpu_node {
    pub bounds_min: [f32; 3],
    pub bounds_max: [f32; 3],
    pub primitive_count: u32,
    pub left_first: u32,
}

#[repr(C)]
#[derive(Copy, Clone, Debug, Default)]
pub struct bvhgpu_triangle {
    pub vertices: [f32; 9],
}

#[repr(C)]
#[derive(Copy, Clone, Debug, Default)]
pub struct bvhgpu_ray {
    pub origin: [f32; 3],
    pub t: f32,
    pub direction: [f32; 3],
    pub reserved: u32,
}

#[repr(C)]
#[derive(Copy, Clone, Debug, Default)]
pub struct bvhgpu_hit {
    pub t: f32,
    pub u: f32,
    pub v: f32,
    pub prim: u32,
    pub inst: u32,
}

#[repr(C)]
#[derive(Copy, Clone, Debug, Default)]
pub struct bvhgpu_tlas_node {
    pub bounds_min: [f32; 3],
    pub bounds_max: [f32; 3],
    pub left_right: u32,
    pub blas: u32,
}

#[repr(C)]
#[derive(Copy, Clone, Debug, Default)]
pub struct bvhgpu_camera {
    pub top_left: [f32; 3],
    pub top_right: [f32; 3],
    pub bottom_left: [f32; 3],
    pub view_inv: [f32; 16],
}

#[repr(C)]
#[derive(Copy, Clone, Debug, Default)]
pub struct bvhgpu_batch_item {
    pub blas: u32,
    pub ray_offset: u32,
    pub ray_count: u32,
    pub reserved: u32,
}

#[repr(C)]
#[derive(Copy, Clone, Debug, Default)]
pub struct bvhgpu_tune_config {
    pub block: u32,
    pub min_blocks: u32,
    pub stack: u32,
    pub big_leaf: u32,
    pub refill: u32,
    pub hidden: u32,
}

#[repr(C)]
#[derive(Copy, Clone, Debug)]
pub struct bvhgpu_tune_job {
    pub kernel: c_int,
    pub target: u32,
    pub d_rays: *const bvhgpu_ray,
    pub n: u32,
    pub seed: u32,
    pub d_hits0: *mut bvhgpu_hit,
    pub d_hits1: *mut bvhgpu_hit,
    pub items: *const bvhgpu_batch_item,
    pub nitems: u32,
}

#[repr(C)]
#[derive(Copy, Clone, Debug, Default)]
pub struct bvhgpu_rigid_body {
    pub inverse_mass: f32,
    pub inverse_inertia: [f32; 9],
    pub linear_drag: f32,
    pub angular_drag: f32,
    pub position: [f32; 3],
    pub orientation: [f32; 4],
    pub velocity: [f32; 3],
    pub rotation: [f32; 3],
    pub inverse_inertia_world: [f32; 9],
    pub motion: f32,
    pub is_awake: u32,
    pub can_sleep: u32,
    pub transform: [f32; 16],
    pub force_accum: [f32; 3],
    pub torque_accum: [f32; 3],
    pub acceleration: [f32; 3],
    pub last_frame_acceleration: [f32; 3],
}

#[repr(C)]
#[derive(Copy, Clone, Debug, Default)]
pub struct bvhgpu_force_generator {
    pub kind: u32,
    pub body: u32,
    pub other: u32,
    pub reserved: u32,
    pub gravity: [f32; 3],
    pub spring_point: [f32; 3],
    pub other_point: [f32; 3],
    pub spring_constant: f32,
    pub rest_length: f32,
}

impl Default for bvhgpu_tune_job {
    fn default() -> Self {
        Self { kernel: 0, target: 0, d_rays: core::ptr::null(), n: 0, seed: 0,
               d_hits0: core::ptr::null_mut(), d_hits1: core::ptr::null_mut(),
               items: core::ptr::null(), nitems: 0 }
    }
}

extern "C" {
    pub fn bvhgpu_create(out: *mut *mut bvhgpu_ctx, device: c_int) -> c_int;
    pub fn bvhgpu_destroy(ctx: *mut bvhgpu_ctx) -> c_int;
    pub fn bvhgpu_last_error(ctx: *const bvhgpu_ctx) -> *const c_char;
    pub fn bvhgpu_launch_count() -> u64;
    pub fn bvhgpu_sync(ctx: *mut bvhgpu_ctx) -> c_int;
    pub fn bvhgpu_get_stream(ctx: *mut bvhgpu_ctx) -> bvhgpu_stream;
    pub fn bvhgpu_set_deadline(ctx: *mut bvhgpu_ctx, ns: u64) -> c_int;
    pub fn bvhgpu_device_alloc(ctx: *mut bvhgpu_ctx, bytes: usize, out: *mut *mut c_void) -> c_int;
    pub fn bvhgpu_device_free(ctx: *mut bvhgpu_ctx, p: *mut c_void) -> c_int;
    pub fn bvhgpu_host_alloc(ctx: *mut bvhgpu_ctx, bytes: usize, out: *mut *mut c_void) -> c_int;
    pub fn bvhgpu_host_free(ctx: *mut bvhgpu_ctx, p: *mut c_void) -> c_int;
    pub fn bvhgpu_copy_to_device(ctx: *mut bvhgpu_ctx, dst: *mut c_void, src: *const c_void, bytes: usize, s: bvhgpu_stream) -> c_int;
    pub fn bvhgpu_copy_to_host(ctx: *mut bvhgpu_ctx, dst: *mut c_void, src: *const c_void, bytes: usize, s: bvhgpu_stream) -> c_int;
    pub fn bvhgpu_memset_device(ctx: *mut bvhgpu_ctx, dst: *mut c_void, value: c_int, bytes: usize, s: bvhgpu_stream) -> c_int;
    pub fn bvhgpu_flush_l2(ctx: *mut bvhgpu_ctx, s: bvhgpu_stream) -> c_int;
    pub fn bvhgpu_event_create(ctx: *mut bvhgpu_ctx, ev: *mut *mut c_void) -> c_int;
    pub fn bvhgpu_event_destroy(ctx: *mut bvhgpu_ctx, ev: *mut c_void) -> c_int;
    pub fn bvhgpu_event_record(ctx: *mut bvhgpu_ctx, ev: *mut c_void, s: bvhgpu_stream) -> c_int;
    pub fn bvhgpu_event_elapsed_ms(ctx: *mut bvhgpu_ctx, start: *mut c_void, stop: *mut c_void, ms: *mut f32) -> c_int;
    pub fn bvhgpu_profile_enable(ctx: *mut bvhgpu_ctx, enable: c_int) -> c_int;
    pub fn bvhgpu_profile_read(ctx: *mut bvhgpu_ctx, ms: *mut f64, launches: *mut u64) -> c_int;
    pub fn bvhgpu_build_bvh_device(ctx: *mut bvhgpu_ctx, mesh: *mut bvhgpu_triangle, n: u32, nodes_out: *mut bvhgpu_node, nodes_used: *mut u32, perm_out: *mut u32) -> c_int;
    pub fn bvhgpu_blas_build(ctx: *mut bvhgpu_ctx, mesh: *mut bvhgpu_triangle, n: u32, blas_id: *mut u32) -> c_int;
    pub fn bvhgpu_mesh_decode(text: *const c_char, len: usize, format: c_int, tris: *mut bvhgpu_triangle, normals: *mut f32, uvs: *mut f32, cap: u32, ntris: *mut u32, err: *mut c_char, errlen: usize) -> c_int;
    pub fn bvhgpu_mesh_decode_file(path: *const c_char, format: c_int, tris: *mut bvhgpu_triangle, normals: *mut f32, uvs: *mut f32, cap: u32, ntris: *mut u32, err: *mut c_char, errlen: usize) -> c_int;
    pub fn bvhgpu_triangles_intersect(ctx: *mut bvhgpu_ctx, tris: *const bvhgpu_triangle, ntris: u32, rays: *const bvhgpu_ray, n: u32, mode: c_int, hits: *mut bvhgpu_hit) -> c_int;
    pub fn bvhgpu_triangles_intersect_async(ctx: *mut bvhgpu_ctx, d_tris: *const bvhgpu_triangle, ntris: u32, d_rays: *const bvhgpu_ray, n: u32, mode: c_int, d_hits: *mut bvhgpu_hit, s: bvhgpu_stream) -> c_int;
    pub fn bvhgpu_build_bvh_host(mesh: *mut bvhgpu_triangle, n: u32, nodes_out: *mut bvhgpu_node, nodes_used: *mut u32) -> c_int;
    pub fn bvhgpu_build_bvh_host_indexed(mesh: *mut bvhgpu_triangle, n: u32, nodes_out: *mut bvhgpu_node, nodes_used: *mut u32, perm_out: *mut u32) -> c_int;
    pub fn bvhgpu_blas_upload(ctx: *mut bvhgpu_ctx, nodes: *const bvhgpu_node, nodes_used: u32, tris: *const bvhgpu_triangle, ntris: u32, blas_id: *mut u32) -> c_int;
    pub fn bvhgpu_blas_free(ctx: *mut bvhgpu_ctx, blas_id: u32) -> c_int;
    pub fn bvhgpu_blas_info(ctx: *mut bvhgpu_ctx, blas_id: u32, nodes_used: *mut u32, ntris: *mut u32, depth: *mut u32) -> c_int;
    pub fn bvhgpu_blas_hidden(ctx: *mut bvhgpu_ctx, blas_id: u32, nodes: *mut u32, pairs: *mut u32, depth: *mut u32) -> c_int;
    pub fn bvhgpu_blas_hidden_download(ctx: *mut bvhgpu_ctx, blas_id: u32, nodes: *mut f32, cones: *mut f32, slots: *mut u32, table: *mut u32, ncones: *mut u32) -> c_int;
    pub fn bvhgpu_blas_trace_counts(ctx: *mut bvhgpu_ctx, blas_id: u32, d_rays: *const bvhgpu_ray, n: u32, d_hits: *mut bvhgpu_hit, counts: *mut u64) -> c_int;
    pub fn bvhgpu_blas_update_vertices(ctx: *mut bvhgpu_ctx, blas_id: u32, tris: *const bvhgpu_triangle) -> c_int;
    pub fn bvhgpu_blas_update_vertices_async(ctx: *mut bvhgpu_ctx, blas_id: u32, d_tris: *const bvhgpu_triangle, s: bvhgpu_stream) -> c_int;
    pub fn bvhgpu_blas_refit(ctx: *mut bvhgpu_ctx, blas_id: u32) -> c_int;
    pub fn bvhgpu_blas_refit_async(ctx: *mut bvhgpu_ctx, blas_id: u32, s: bvhgpu_stream) -> c_int;
    pub fn bvhgpu_blas_download_nodes(ctx: *mut bvhgpu_ctx, blas_id: u32, nodes: *mut bvhgpu_node) -> c_int;
    pub fn bvhgpu_blas_intersect(ctx: *mut bvhgpu_ctx, blas_id: u32, rays: *const bvhgpu_ray, n: u32, hits: *mut bvhgpu_hit) -> c_int;
    pub fn bvhgpu_blas_intersect_async(ctx: *mut bvhgpu_ctx, blas_id: u32, d_rays: *const bvhgpu_ray, n: u32, d_hits: *mut bvhgpu_hit, s: bvhgpu_stream) -> c_int;
    pub fn bvhgpu_blas_trace_bounce(ctx: *mut bvhgpu_ctx, blas_id: u32, rays: *const bvhgpu_ray, n: u32, seed: u32, mode: c_int, hits0: *mut bvhgpu_hit, hits1: *mut bvhgpu_hit, n_bounce: *mut u32) -> c_int;
    pub fn bvhgpu_blas_trace_bounce_async(ctx: *mut bvhgpu_ctx, blas_id: u32, d_rays: *const bvhgpu_ray, n: u32, seed: u32, mode: c_int, d_hits0: *mut bvhgpu_hit, d_hits1: *mut bvhgpu_hit, s: bvhgpu_stream) -> c_int;
    pub fn bvhgpu_blas_bounce_rays(ctx: *mut bvhgpu_ctx, blas_id: u32, rays: *const bvhgpu_ray, n: u32, seed: u32, out: *mut bvhgpu_ray, valid: *mut u8) -> c_int;
    pub fn bvhgpu_trace_batch(ctx: *mut bvhgpu_ctx, items: *const bvhgpu_batch_item, nitems: u32, rays: *const bvhgpu_ray, nrays: u32, mode: c_int, hits: *mut bvhgpu_hit) -> c_int;
    pub fn bvhgpu_trace_batch_async(ctx: *mut bvhgpu_ctx, items: *const bvhgpu_batch_item, nitems: u32, d_rays: *const bvhgpu_ray, nrays: u32, mode: c_int, d_hits: *mut bvhgpu_hit, s: bvhgpu_stream) -> c_int;
    pub fn bvhgpu_scene_create(ctx: *mut bvhgpu_ctx, blas_ids: *const u32, nobjects: u32, scene_id: *mut u32) -> c_int;
    pub fn bvhgpu_scene_free(ctx: *mut bvhgpu_ctx, scene_id: u32) -> c_int;
    pub fn bvhgpu_scene_set_transforms(ctx: *mut bvhgpu_ctx, scene_id: u32, xf: *const f32, inv: *const f32) -> c_int;
    pub fn bvhgpu_scene_set_transforms_async(ctx: *mut bvhgpu_ctx, scene_id: u32, d_xf: *const f32, d_inv: *const f32, s: bvhgpu_stream) -> c_int;
    pub fn bvhgpu_scene_rebuild(ctx: *mut bvhgpu_ctx, scene_id: u32) -> c_int;
    pub fn bvhgpu_scene_rebuild_async(ctx: *mut bvhgpu_ctx, scene_id: u32, s: bvhgpu_stream) -> c_int;
    pub fn bvhgpu_scene_download_tlas(ctx: *mut bvhgpu_ctx, scene_id: u32, nodes: *mut bvhgpu_tlas_node, nodes_used: *mut u32) -> c_int;
    pub fn bvhgpu_scene_intersect(ctx: *mut bvhgpu_ctx, scene_id: u32, rays: *const bvhgpu_ray, n: u32, hits: *mut bvhgpu_hit) -> c_int;
    pub fn bvhgpu_scene_intersect_async(ctx: *mut bvhgpu_ctx, scene_id: u32, d_rays: *const bvhgpu_ray, n: u32, d_hits: *mut bvhgpu_hit, s: bvhgpu_stream) -> c_int;
    pub fn bvhgpu_scene_trace_bounce_async(ctx: *mut bvhgpu_ctx, scene_id: u32, d_rays: *const bvhgpu_ray, n: u32, seed: u32, d_hits0: *mut bvhgpu_hit, d_hits1: *mut bvhgpu_hit, s: bvhgpu_stream) -> c_int;
    pub fn bvhgpu_scene_bounce_rays(ctx: *mut bvhgpu_ctx, scene_id: u32, rays: *const bvhgpu_ray, n: u32, seed: u32, out: *mut bvhgpu_ray, valid: *mut u8) -> c_int;
    pub fn bvhgpu_scene_download_transforms(ctx: *mut bvhgpu_ctx, scene_id: u32, xf: *mut f32, inv: *mut f32) -> c_int;
    pub fn bvhgpu_mesh_wobble_async(ctx: *mut bvhgpu_ctx, mesh_id: u32, d_dirs: *const f32, d_r0: *const f32, d_phase: *const f32, amp: f32, freq: f32, d_time: *const f32, s: bvhgpu_stream) -> c_int;
    pub fn bvhgpu_scene_animate_async(ctx: *mut bvhgpu_ctx, scene_id: u32, d_rot0: *const f32, d_axis: *const f32, d_omega: *const f32, d_scale: *const f32, d_trans: *const f32, d_time: *const f32, s: bvhgpu_stream) -> c_int;
    pub fn bvhgpu_advance_time_async(ctx: *mut bvhgpu_ctx, d_time: *mut f32, dt: f32, s: bvhgpu_stream) -> c_int;
    pub fn bvhgpu_graph_begin(ctx: *mut bvhgpu_ctx) -> c_int;
    pub fn bvhgpu_graph_end(ctx: *mut bvhgpu_ctx, graph_id: *mut u32) -> c_int;
    pub fn bvhgpu_graph_launch(ctx: *mut bvhgpu_ctx, graph_id: u32) -> c_int;
    pub fn bvhgpu_graph_free(ctx: *mut bvhgpu_ctx, graph_id: u32) -> c_int;
    pub fn bvhgpu_render(ctx: *mut bvhgpu_ctx, blas_id: u32, camera: *const bvhgpu_camera, width: c_int, height: c_int, accumulator: c_int, acc_params: *const f32, shader: c_int, shader_params: *const f32, normals: *const f32, rgba: *mut u8, rays_traced: *mut u64) -> c_int;
    pub fn bvhgpu_render_textured(ctx: *mut bvhgpu_ctx, blas_id: u32, camera: *const bvhgpu_camera, width: c_int, height: c_int, tex_coords: *const f32, texels: *const u8, tex_w: u32, tex_h: u32, shader: c_int, shader_params: *const f32, rgba: *mut u8, rays_traced: *mut u64) -> c_int;
    pub fn bvhgpu_blas_set_shading(ctx: *mut bvhgpu_ctx, blas_id: u32, normals: *const f32, tex_coords: *const f32, texels: *const u8, tex_w: u32, tex_h: u32) -> c_int;
    pub fn bvhgpu_render_scene(ctx: *mut bvhgpu_ctx, scene_id: u32, camera: *const bvhgpu_camera, width: c_int, height: c_int, accumulator: c_int, acc_params: *const f32, shader: c_int, shader_params: *const f32, lookup: c_int, rgba: *mut u8, rays_traced: *mut u64) -> c_int;
    pub fn bvhgpu_mesh_create(ctx: *mut bvhgpu_ctx, blas_id: u32, faces: *const u32, nfaces: u32, verts: *const f32, vnormals: *const f32, nverts: u32, mesh_id: *mut u32) -> c_int;
    pub fn bvhgpu_mesh_free(ctx: *mut bvhgpu_ctx, mesh_id: u32) -> c_int;
    pub fn bvhgpu_mesh_vertices(ctx: *mut bvhgpu_ctx, mesh_id: u32, d_verts: *mut *mut f32) -> c_int;
    pub fn bvhgpu_mesh_set_vertices(ctx: *mut bvhgpu_ctx, mesh_id: u32, verts: *const f32) -> c_int;
    pub fn bvhgpu_mesh_update_async(ctx: *mut bvhgpu_ctx, mesh_id: u32, s: bvhgpu_stream) -> c_int;
    pub fn bvhgpu_lambert_forward_async(ctx: *mut bvhgpu_ctx, mesh_id: u32, d_rays: *const bvhgpu_ray, n: u32, light: *const f32, d_image: *mut f32, d_hits: *mut bvhgpu_hit, s: bvhgpu_stream) -> c_int;
    pub fn bvhgpu_mse_loss(ctx: *mut bvhgpu_ctx, d_image: *const f32, d_target: *const f32, n: u32, loss: *mut f64) -> c_int;
    pub fn bvhgpu_lambert_adjoint_async(ctx: *mut bvhgpu_ctx, mesh_id: u32, d_rays: *const bvhgpu_ray, n: u32, light: *const f32, d_hits: *const bvhgpu_hit, d_image: *const f32, d_target: *const f32, d_grad: *mut f32, s: bvhgpu_stream) -> c_int;
    pub fn bvhgpu_mesh_sgd_step_async(ctx: *mut bvhgpu_ctx, mesh_id: u32, d_grad: *mut f32, lr: f32, s: bvhgpu_stream) -> c_int;
    pub fn bvhgpu_tune_get(ctx: *mut bvhgpu_ctx, kernel: c_int, out: *mut bvhgpu_tune_config) -> c_int;
    pub fn bvhgpu_tune_set(ctx: *mut bvhgpu_ctx, kernel: c_int, cfg: *const bvhgpu_tune_config) -> c_int;
    pub fn bvhgpu_tune_space(kernel: c_int, out: *mut bvhgpu_tune_config, cap: u32, count: *mut u32) -> c_int;
    pub fn bvhgpu_autotune(ctx: *mut bvhgpu_ctx, job: *const bvhgpu_tune_job, reps: u32, best: *mut bvhgpu_tune_config, best_ms: *mut f32) -> c_int;
    pub fn bvhgpu_world_create(ctx: *mut bvhgpu_ctx, bodies: *const bvhgpu_rigid_body, nbodies: u32, gens: *const bvhgpu_force_generator, ngens: u32, world_id: *mut u32) -> c_int;
    pub fn bvhgpu_world_free(ctx: *mut bvhgpu_ctx, world_id: u32) -> c_int;
    pub fn bvhgpu_world_start_frame_async(ctx: *mut bvhgpu_ctx, world_id: u32, s: bvhgpu_stream) -> c_int;
    pub fn bvhgpu_world_step_async(ctx: *mut bvhgpu_ctx, world_id: u32, dt: f32, s: bvhgpu_stream) -> c_int;
    pub fn bvhgpu_world_download(ctx: *mut bvhgpu_ctx, world_id: u32, bodies_out: *mut bvhgpu_rigid_body) -> c_int;
    pub fn bvhgpu_scene_bind_world(ctx: *mut bvhgpu_ctx, scene_id: u32, world_id: u32, body_of: *const u32, transform_init: *const f32) -> c_int;
    pub fn bvhgpu_scene_run_async(ctx: *mut bvhgpu_ctx, scene_id: u32, dt: f32, s: bvhgpu_stream) -> c_int;
    pub fn bvhgpu_refit_noalloc(d_nodes: *mut bvhgpu_node, nodes_used: u32, d_tris: *const bvhgpu_triangle, ntris: u32, stream: bvhgpu_stream, d_status: *mut u32) -> c_int;
}
