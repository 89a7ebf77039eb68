//! A GPU `Integrator` for the bvhtracer crate and safe wrappers over `bvhgpu-sys`.
//!
//! `GpuIntegrator` is installed where the reference installs its CPU `PathTracer`:
//! `Renderer::new(Box::new(GpuIntegrator::new(...)?))` (bvhtracer/src/renderer.rs:392-395).  Each
//! `evaluate(state, scene)` (renderer.rs:104-106) mirrors the scene on the GPU -- one BLAS per
//! distinct model (the model's own SAH-built node array and triangles, uploaded as-is), one object
//! per scene object with its transform and cached inverse -- rebuilds the TLAS, renders every
//! pixel through `bvhgpu_render_scene` (the TLAS with instance transforms, as `Scene::intersect`
//! does) and writes the RGBA8 frame into the renderer's frame buffer.  Images are identical to the
//! CPU `PathTracer`'s with the same accumulator and shader.
//!
//! The reference crate keeps a few things private that this needs; INTEGRATION.md lists the
//! read-only accessors a maintainer adds (`Scene::len`, `Model::bvh`, `Bvh::export_nodes`,
//! `FrameBuffer::as_bytes_mut`, `TextureMaterial::texels`).  Neither the accessors nor this crate
//! change the reference's own results.
use std::ffi::CStr;
use std::fmt;
use std::os::raw::c_int;
use std::rc::Rc;

use bvhgpu_sys as sys;
use bvhtracer::{Integrator, RendererState, Scene};

/// A status other than BVHGPU_OK, with the library's message.
#[derive(Debug, Clone)]
pub struct GpuError {
    pub code: i32,
    pub message: String,
}

impl fmt::Display for GpuError {
    fn fmt(&self, f: &mut fmt::Formatter<'_>) -> fmt::Result {
        write!(f, "bvhgpu error {}: {}", self.code, self.message)
    }
}

impl std::error::Error for GpuError {}

/// One bvhgpu context on one CUDA device.  Not `Send`: like the reference's `Rc<RefCell<Model>>`
/// ownership, a context belongs to one host thread.
pub struct Context {
    raw: *mut sys::bvhgpu_ctx,
}

impl Context {
    pub fn new(device: i32) -> Result<Self, GpuError> {
        let mut raw = std::ptr::null_mut();
        let rc = unsafe { sys::bvhgpu_create(&mut raw, device) };
        if rc != sys::BVHGPU_OK {
            return Err(GpuError { code: rc, message: "bvhgpu_create failed (no usable CUDA device?)".into() });
        }
        Ok(Self { raw })
    }

    fn check(&self, rc: c_int) -> Result<(), GpuError> {
        if rc == sys::BVHGPU_OK {
            return Ok(());
        }
        let msg = unsafe { sys::bvhgpu_last_error(self.raw) };
        let message = if msg.is_null() {
            String::new()
        } else {
            unsafe { CStr::from_ptr(msg) }.to_string_lossy().into_owned()
        };
        Err(GpuError { code: rc, message })
    }

    pub fn raw(&self) -> *mut sys::bvhgpu_ctx {
        self.raw
    }

    /// Uploads a BVH built by the reference's `BvhBuilder` (node array in its 32-byte layout) with
    /// its triangles; returns the BLAS id.
    pub fn upload_blas(&mut self, nodes: &[sys::bvhgpu_node], tris: &[sys::bvhgpu_triangle]) -> Result<u32, GpuError> {
        let mut id = 0u32;
        let rc = unsafe {
            sys::bvhgpu_blas_upload(self.raw, nodes.as_ptr(), nodes.len() as u32, tris.as_ptr(), tris.len() as u32, &mut id)
        };
        self.check(rc).map(|_| id)
    }

    /// New vertex positions (same triangle order) followed by `Bvh::refit` on the device.
    pub fn update_and_refit(&mut self, blas: u32, tris: &[sys::bvhgpu_triangle]) -> Result<(), GpuError> {
        self.check(unsafe { sys::bvhgpu_blas_update_vertices(self.raw, blas, tris.as_ptr()) })?;
        self.check(unsafe { sys::bvhgpu_blas_refit(self.raw, blas) })
    }

    /// The model's normals (9 floats per triangle), texture coordinates (6 per triangle) and RGB8
    /// texture for the normal / texture accumulators.
    pub fn set_shading(&mut self, blas: u32, normals: Option<&[f32]>, tex_coords: Option<&[f32]>,
                       texture: Option<(&[u8], u32, u32)>) -> Result<(), GpuError> {
        let (texels, w, h) = match texture {
            Some((t, w, h)) => (t.as_ptr(), w, h),
            None => (std::ptr::null(), 0, 0),
        };
        let rc = unsafe {
            sys::bvhgpu_blas_set_shading(self.raw, blas, normals.map_or(std::ptr::null(), |n| n.as_ptr()),
                                         tex_coords.map_or(std::ptr::null(), |t| t.as_ptr()), texels, w, h)
        };
        self.check(rc)
    }

    pub fn free_blas(&mut self, blas: u32) -> Result<(), GpuError> {
        self.check(unsafe { sys::bvhgpu_blas_free(self.raw, blas) })
    }

    pub fn free_scene(&mut self, scene: u32) -> Result<(), GpuError> {
        self.check(unsafe { sys::bvhgpu_scene_free(self.raw, scene) })
    }

    pub fn create_scene(&mut self, blas_of_object: &[u32]) -> Result<u32, GpuError> {
        let mut id = 0u32;
        let rc = unsafe { sys::bvhgpu_scene_create(self.raw, blas_of_object.as_ptr(), blas_of_object.len() as u32, &mut id) };
        self.check(rc).map(|_| id)
    }

    /// `SceneObject::set_transform` for every object (column-major transforms and cached inverses)
    /// and `Scene::rebuild` (the TLAS).
    pub fn set_transforms_and_rebuild(&mut self, scene: u32, xf: &[[f32; 16]], inv: &[[f32; 16]]) -> Result<(), GpuError> {
        assert_eq!(xf.len(), inv.len());
        let rc = unsafe { sys::bvhgpu_scene_set_transforms(self.raw, scene, xf.as_ptr() as *const f32, inv.as_ptr() as *const f32) };
        self.check(rc)?;
        self.check(unsafe { sys::bvhgpu_scene_rebuild(self.raw, scene) })
    }

    /// `Scene::intersect` for a batch of rays.
    pub fn scene_intersect(&mut self, scene: u32, rays: &[sys::bvhgpu_ray], hits: &mut [sys::bvhgpu_hit]) -> Result<(), GpuError> {
        assert_eq!(rays.len(), hits.len());
        let rc = unsafe { sys::bvhgpu_scene_intersect(self.raw, scene, rays.as_ptr(), rays.len() as u32, hits.as_mut_ptr()) };
        self.check(rc)
    }

    /// Primaries + one diffuse bounce per hit in one persistent launch (`bvhgpu_blas_trace_bounce`).
    /// `rays` and the hit slices are read and written in place when the GPU can (page-locked memory,
    /// or ordinary memory on a Grace-attached GPU); returns the number of bounce rays traced.
    pub fn trace_bounce(&mut self, blas: u32, rays: &[sys::bvhgpu_ray], seed: u32, hits0: &mut [sys::bvhgpu_hit],
                        hits1: &mut [sys::bvhgpu_hit]) -> Result<u32, GpuError> {
        assert!(hits0.len() == rays.len() && hits1.len() == rays.len());
        let mut n_bounce = 0u32;
        let rc = unsafe {
            sys::bvhgpu_blas_trace_bounce(self.raw, blas, rays.as_ptr(), rays.len() as u32, seed,
                                          sys::BVHGPU_MODE_PERSISTENT, hits0.as_mut_ptr(), hits1.as_mut_ptr(),
                                          &mut n_bounce)
        };
        self.check(rc).map(|_| n_bounce)
    }

    /// A time budget for each persistent launch of this context (0: none).  A launch past it returns
    /// `GpuError { code: BVHGPU_ERR_DEADLINE, .. }` with its outputs incomplete; the context stays usable.
    pub fn set_deadline(&mut self, budget: std::time::Duration) -> Result<(), GpuError> {
        let ns = u64::try_from(budget.as_nanos()).unwrap_or(u64::MAX);
        self.check(unsafe { sys::bvhgpu_set_deadline(self.raw, ns) })
    }

    /// `PathTracer::evaluate` over a scene into `rgba` (width * height * 4 bytes); returns the rays traced.
    #[allow(clippy::too_many_arguments)]
    pub fn render_scene(&mut self, scene: u32, camera: &sys::bvhgpu_camera, width: usize, height: usize,
                        accumulator: &Accumulator, shader: &Shader, lookup: Lookup, rgba: &mut [u8]) -> Result<u64, GpuError> {
        assert_eq!(rgba.len(), width * height * 4);
        let (acc, acc_params) = accumulator.raw();
        let (sh, sh_params) = shader.raw();
        let mut rays = 0u64;
        let rc = unsafe {
            sys::bvhgpu_render_scene(self.raw, scene, camera, width as c_int, height as c_int, acc, acc_params.as_ptr(),
                                     sh, sh_params.as_ptr(), lookup as c_int, rgba.as_mut_ptr(), &mut rays)
        };
        self.check(rc).map(|_| rays)
    }
}

impl Drop for Context {
    fn drop(&mut self) {
        unsafe {
            sys::bvhgpu_destroy(self.raw);
        }
    }
}

/// The accumulators of renderer.rs:134-334.
#[derive(Clone, Debug)]
pub enum Accumulator {
    /// IntersectionAccumulator(hit, miss)
    Intersection([f32; 3], [f32; 3]),
    Depth,
    UvMapping,
    NormalMapping,
    TextureMaterial,
}

impl Accumulator {
    fn raw(&self) -> (c_int, Vec<f32>) {
        match self {
            Accumulator::Intersection(h, m) => (sys::BVHGPU_ACC_INTERSECTION, vec![h[0], h[1], h[2], m[0], m[1], m[2]]),
            Accumulator::Depth => (sys::BVHGPU_ACC_DEPTH, vec![0.0; 6]),
            Accumulator::UvMapping => (sys::BVHGPU_ACC_UV, vec![0.0; 6]),
            Accumulator::NormalMapping => (sys::BVHGPU_ACC_NORMAL, vec![0.0; 6]),
            Accumulator::TextureMaterial => (sys::BVHGPU_ACC_TEXTURE, vec![0.0; 6]),
        }
    }
}

/// The pixel shaders of renderer.rs:116-222.
#[derive(Clone, Debug)]
pub enum Shader {
    RadianceToRgb,
    /// IntersectionShader(hit rgba, miss rgba)
    Intersection([u8; 4], [u8; 4]),
    /// DepthMappingShader(scale, offset)
    DepthMapping(f32, f32),
}

impl Shader {
    fn raw(&self) -> (c_int, Vec<f32>) {
        match self {
            Shader::RadianceToRgb => (sys::BVHGPU_SHADER_RADIANCE, vec![0.0; 8]),
            Shader::Intersection(h, m) => (sys::BVHGPU_SHADER_INTERSECTION,
                                           h.iter().chain(m.iter()).map(|&c| c as f32).collect()),
            Shader::DepthMapping(s, o) => (sys::BVHGPU_SHADER_DEPTH, vec![*s, *o, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0]),
        }
    }
}

/// Which model the normal / texture accumulators read for a hit (see bvhgpu_render_scene).
#[derive(Clone, Copy, Debug, PartialEq, Eq)]
#[repr(i32)]
pub enum Lookup {
    /// What the reference computes: object 0's model and transform (its hits carry instance 0).
    Reference = sys::BVHGPU_LOOKUP_REFERENCE,
    /// The hit's own object.
    HitObject = sys::BVHGPU_LOOKUP_HIT_OBJECT,
}

fn matrix16<T>(m: &T) -> [f32; 16] {
    // Transform3<f32> (repr(transparent)) and Matrix4x4<f32> are 16 column-major f32.
    assert_eq!(std::mem::size_of::<T>(), 64);
    unsafe { *(m as *const T as *const [f32; 16]) }
}

fn camera_of(scene: &Scene) -> sys::bvhgpu_camera {
    let cam = scene.active_camera();
    let (tl, tr, bl) = (cam.top_left_eye(), cam.top_right_eye(), cam.bottom_left_eye());
    sys::bvhgpu_camera {
        top_left: [tl.x, tl.y, tl.z],
        top_right: [tr.x, tr.y, tr.z],
        bottom_left: [bl.x, bl.y, bl.z],
        view_inv: matrix16(cam.view_matrix_inv()),
    }
}

/// GPU handles of the scene last rendered: a BLAS per distinct model, a scene over the objects.
struct Mirror {
    models: Vec<*const ()>,  // Rc identity of each object's model, object order
    blases: Vec<u32>,        // one per distinct model
    scene: u32,
}

/// The GPU `Integrator` (renderer.rs:104-106): renders the whole `Scene` through the TLAS.
pub struct GpuIntegrator {
    ctx: Context,
    accumulator: Accumulator,
    shader: Shader,
    lookup: Lookup,
    mirror: Option<Mirror>,
    models_dirty: bool,
    rgba: Vec<u8>,
}

impl GpuIntegrator {
    /// The accumulator and shader the `RendererState` holds (its trait objects are opaque, so they
    /// are named here again).
    pub fn new(device: i32, accumulator: Accumulator, shader: Shader, lookup: Lookup) -> Result<Self, GpuError> {
        Ok(Self { ctx: Context::new(device)?, accumulator, shader, lookup, mirror: None, models_dirty: false,
                  rgba: Vec::new() })
    }

    /// Call after changing model vertices on the host (e.g. after `ModelInstance::refit`): the next
    /// frame re-uploads every model's triangles and refits its BLAS on the device.
    pub fn set_models_dirty(&mut self) {
        self.models_dirty = true;
    }

    pub fn context(&mut self) -> &mut Context {
        &mut self.ctx
    }

    fn sync_scene(&mut self, scene: &Scene) -> Result<u32, GpuError> {
        let n = scene.len();
        let mut models: Vec<*const ()> = Vec::with_capacity(n);
        for i in 0..n {
            models.push(Rc::as_ptr(&scene.get_unchecked(i).model().model()) as *const ());
        }
        let current = self.mirror.as_ref().map_or(false, |m| m.models == models);
        if !current || self.models_dirty {
            if let Some(old) = self.mirror.take() {
                self.ctx.free_scene(old.scene)?;
                for b in old.blases {
                    self.ctx.free_blas(b)?;
                }
            }
            let mut distinct: Vec<*const ()> = Vec::new();
            let mut blas_ids: Vec<u32> = Vec::new();
            let mut blas_of: Vec<u32> = Vec::with_capacity(n);
            for i in 0..n {
                let key = models[i];
                let k = match distinct.iter().position(|&d| d == key) {
                    Some(k) => k,
                    None => {
                        let rc_model = scene.get_unchecked(i).model().model();
                        let model = rc_model.borrow();
                        let tris: &[sys::bvhgpu_triangle] = unsafe {
                            // Triangle<f32> is repr(C) over three Vector3<f32>: 36 bytes, the ABI's layout
                            std::slice::from_raw_parts(model.primitives().as_ptr() as *const sys::bvhgpu_triangle,
                                                       model.primitives().len())
                        };
                        let nodes: Vec<sys::bvhgpu_node> = model.bvh().export_nodes().iter().map(|w| sys::bvhgpu_node {
                            bounds_min: [f32::from_bits(w[0]), f32::from_bits(w[1]), f32::from_bits(w[2])],
                            bounds_max: [f32::from_bits(w[3]), f32::from_bits(w[4]), f32::from_bits(w[5])],
                            primitive_count: w[6],
                            left_first: w[7],
                        }).collect();
                        let id = self.ctx.upload_blas(&nodes, tris)?;
                        let normals: Vec<f32> = model.normals().iter()
                            .flat_map(|n| (0..3).flat_map(move |c| [n[c].x, n[c].y, n[c].z]))
                            .collect();
                        let tex_coords: Vec<f32> = model.tex_coords().iter()
                            .flat_map(|t| (0..3).flat_map(move |c| [t[c].x, t[c].y]))
                            .collect();
                        let (texels, w, h) = model.texture().texels();
                        self.ctx.set_shading(id, Some(&normals), Some(&tex_coords), Some((texels, w as u32, h as u32)))?;
                        distinct.push(key);
                        blas_ids.push(id);
                        distinct.len() - 1
                    }
                };
                blas_of.push(blas_ids[k]);
            }
            let id = self.ctx.create_scene(&blas_of)?;
            self.mirror = Some(Mirror { models, blases: blas_ids, scene: id });
            self.models_dirty = false;
        }
        let mut xf = Vec::with_capacity(n);
        let mut inv = Vec::with_capacity(n);
        for i in 0..n {
            let obj = scene.get_unchecked(i);
            xf.push(matrix16(obj.get_transform()));
            inv.push(matrix16(obj.get_transform_inv()));
        }
        let scene_id = self.mirror.as_ref().map(|m| m.scene).unwrap_or(0);
        self.ctx.set_transforms_and_rebuild(scene_id, &xf, &inv)?;
        Ok(scene_id)
    }

    /// One frame into `rgba` (row-major RGBA8, width * height * 4 bytes).
    pub fn render(&mut self, scene: &Scene, width: usize, height: usize, rgba: &mut [u8]) -> Result<u64, GpuError> {
        let id = self.sync_scene(scene)?;
        let camera = camera_of(scene);
        let (acc, sh, lookup) = (self.accumulator.clone(), self.shader.clone(), self.lookup);
        self.ctx.render_scene(id, &camera, width, height, &acc, &sh, lookup, rgba)
    }
}

impl Integrator for GpuIntegrator {
    fn evaluate(&mut self, state: &mut RendererState, scene: &Scene) -> usize {
        let (w, h) = state.frame_buffer().dimensions();
        let mut frame = std::mem::take(&mut self.rgba);
        frame.resize(w * h * 4, 0);
        let rays = match self.render(scene, w, h, &mut frame) {
            Ok(n) => n as usize,
            // the trait returns a ray count: a failure renders nothing and is reported here
            Err(e) => panic!("GpuIntegrator: {e}"),
        };
        state.frame_buffer_mut().as_bytes_mut().copy_from_slice(&frame);
        self.rgba = frame;
        rays
    }
}
