// Host-side internals of the bvhgpu library: the context, BLAS / scene records and the
// kernel launchers (defined in the kernel translation units, called from api.cu).
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include "../../include/bvhgpu.h"

namespace bvhgpu {

extern std::atomic<uint64_t> g_launches;

// Hidden-tree refresh: pairs per chunk (one warp), and the "none" marker of a group's node / cone.
constexpr uint32_t kRefreshChunk = 256;
constexpr uint32_t kNoRefresh = 0xFFFFFFFFu;
// A chunk's partial result of the refresh's first pass: raw bounds of v0, v0 + e1, v0 + e2, the
// largest |e1_i|, |e2_i|, the sum of the folded unit normals (cone groups), all inputs finite.
struct RefreshAgg {
    float lo[3], hi[3], e1m, e2m, sx, sy, sz;
    bool finite;
};

struct DeviceBlas {
    float4* nodes = nullptr;     // 2 float4 per node (nodes_used nodes)
    float4* tris = nullptr;      // 3 float4 per triangle (v0, e1, e2): traversal layout
    float4* verts = nullptr;     // 3 float4 per triangle (v0, v1, v2): refit input
    ulonglong2* pairs = nullptr; // 5 x 16 bytes per triangle pair: packed traversal layout
    uint32_t* parent = nullptr;  // parent index per node (refit), 0xFFFFFFFF for root/filler
    uint32_t* leaves = nullptr;  // indices of leaf nodes (refit start points)
    uint32_t* counters = nullptr;// refit arrival counters, one per node (kept zeroed)
    uint32_t* tri_leaf = nullptr;        // leaf slot (index into `leaves`) of each triangle, or none
    unsigned long long* leaf_keys = nullptr;  // refit reduction keys, 6 per leaf (kept at identity)
    uint2* hx = nullptr;         // hidden-tree table and pair slots (GBlas::hx), or null
    float4* cones = nullptr;     // hidden-tree cone records (GBlas::cones)
    uint32_t ncones = 0;
    uint4* hwork = nullptr;      // refresh groups: {first pair, end pair, node index or ~0, cone index or ~0}
    uint2* hchunks = nullptr;    // refresh chunks: {group, first pair}, node groups' chunks first
    uint32_t* hchunk0 = nullptr; // first chunk of each group (nwork + 1 entries)
    void* hpart = nullptr;       // per-chunk partial results of the refresh
    uint32_t* harrivals = nullptr;  // per-group arrival counters of the refresh (kept zeroed)
    uint32_t nhid = 0;           // hidden nodes (after the nodes_used reference nodes)
    uint32_t nhp = 0;            // hidden pairs (after the (ntris + 1) / 2 pairs in triangle order)
    uint32_t nwork = 0;          // hidden nodes + cones
    uint32_t nchunks = 0, nbox_chunks = 0;
    uint32_t ref_depth = 0;      // depth of the reference tree (depth adds the hidden trees')
    uint32_t nodes_used = 0;
    uint32_t ntris = 0;
    uint32_t nleaves = 0;
    uint32_t depth = 0;          // traversal depth: reference tree plus the deepest hidden tree
    uint32_t root_count = 0;
    uint32_t root_first = 0;
    // shading data of the BLAS's model (bvhgpu_blas_set_shading), for rendering a scene
    float* normals = nullptr;     // 9 floats per triangle (corner normals), or null
    float* tex_coords = nullptr;  // 6 floats per triangle (corner texture coordinates), or null
    uint8_t* texels = nullptr;    // RGB8 texture, row-major tex_w x tex_h, or null
    uint32_t tex_w = 0, tex_h = 0;
};

// Per entry of a scene's BLAS table: what the normal / texture accumulators read of a model.
struct ShadeEntry {
    const float* normals;
    const float* tex_coords;
    const uint8_t* texels;
    uint32_t tex_w, tex_h, ntris, pad;
};

struct DeviceScene {
    std::vector<uint32_t> blas_ids;  // per object
    uint32_t nobjects = 0;
    float* xf = nullptr;       // 16 per object
    float* inv = nullptr;      // 16 per object
    uint32_t* obj_blas = nullptr;       // per object: index into the scene's BLAS table
    void* blas_table = nullptr;         // GBlas per distinct BLAS used (device)
    uint32_t nblas = 0;
    std::vector<uint32_t> table_blas;   // context BLAS id of each table entry
    float4* tlas = nullptr;    // 2 float4 per TLAS node (2*nobjects nodes)
    void* tlas_work = nullptr; // TLAS rebuild state (40 B per object) above kTlasSharedObjects objects
    uint32_t tlas_nodes_used = 0;
    uint32_t tlas_depth_cap = 0;
    uint32_t world = 0;              // bound physics world (0: none)
    uint32_t* body_of = nullptr;     // per object: body index or 0xFFFFFFFF
    float* transform_init = nullptr; // 16 per object
};

struct DeviceWorld {
    bvhgpu_rigid_body* bodies = nullptr;
    uint32_t nbodies = 0;
    bvhgpu_force_generator* gens = nullptr;  // grouped by body, registry order kept within a body
    uint32_t* gen_off = nullptr;             // nbodies + 1
    uint32_t ngens = 0;
};

// Layout of a mesh's forward-pass schedule (u32 words, for up to `cap` rays): per parity p (the
// pass number's low bit) a flag per ray (1: the next pass serves the ray from its long list) and a
// long list of ray ids; then the counters: the pixel queue, the long list's head, the list sizes
// per parity, the pass number, the ray counts of the last two passes, and whether the last pass
// stopped at a deadline (its flags and list are then incomplete and the next pass ignores them).
struct ForwardSchedule {
    static constexpr uint32_t kQueue = 0, kHead = 1, kCount = 2 /* + parity */, kPass = 4, kRays = 5, kPrevRays = 6,
                              kStopped = 7, kCounters = 8;
    static __host__ __device__ size_t flags(uint32_t cap, uint32_t p) { return (size_t)p * cap; }
    static __host__ __device__ size_t list(uint32_t cap, uint32_t p) { return (size_t)(2u + p) * cap; }
    static __host__ __device__ size_t counters(uint32_t cap) { return 4ull * cap; }
    static size_t words(uint32_t cap) { return 4ull * cap + kCounters; }
};

struct DeviceMesh {
    uint32_t blas = 0;           // BLAS whose triangle i is face i
    uint32_t* faces = nullptr;   // 3 vertex ids per face, in the BLAS's triangle order
    float* verts = nullptr;      // 3 floats per vertex
    float* vnormals = nullptr;   // 3 floats per vertex (fixed shading normals)
    uint32_t nfaces = 0;
    uint32_t nverts = 0;
    uint32_t* sched = nullptr;   // forward-pass schedule (ForwardSchedule), for up to sched_cap rays
    uint32_t sched_cap = 0;
};

struct ProfileRec {
    int kernel;
    cudaEvent_t start, stop;
};

}  // namespace bvhgpu

struct bvhgpu_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    void* host_word = nullptr;  // 64 bytes of pinned host memory for small results
    uint32_t* d_err = nullptr;       // device error flags
    uint32_t* d_scratch = nullptr;   // small device scratch: queue counters etc. (64 words)
    void* l2_flush = nullptr;
    size_t l2_flush_bytes = 0;
    int num_sms = 0;
    int pageable_access = 0;  // kernels may read / write ordinary host memory coherently
    std::string last_error;
    std::map<uint32_t, bvhgpu::DeviceBlas> blas;
    std::map<uint32_t, bvhgpu::DeviceScene> scenes;
    std::map<uint32_t, bvhgpu::DeviceMesh> meshes;
    std::map<uint32_t, bvhgpu::DeviceWorld> worlds;
    uint32_t next_world = 1;
    uint32_t next_blas = 1;
    uint32_t next_scene = 1;
    uint32_t next_mesh = 1;
    double* mse_partials = nullptr;  // per-block partial sums of the loss
    size_t mse_partials_cap = 0;
    // staging buffers for host-pointer entry points (grown on demand)
    void* stage_in = nullptr;
    size_t stage_in_bytes = 0;
    void* stage_out = nullptr;
    size_t stage_out_bytes = 0;
    void* stage_out2 = nullptr;
    size_t stage_out2_bytes = 0;
    // plain-bounce work buffers
    void* bounce_rays = nullptr;     // compacted bounce rays (2 float4 each)
    uint32_t* bounce_pix = nullptr;  // pixel index of each compacted bounce ray
    size_t bounce_cap = 0;
    // persistent batch: device table of the last item list (rebuilt when the items change)
    void* batch_table = nullptr;
    size_t batch_table_bytes = 0;
    std::vector<bvhgpu_batch_item> batch_items;
    uint32_t batch_total = 0;
    uint32_t batch_depth = 1;
    // captured frame graphs
    std::map<uint32_t, std::pair<cudaGraph_t, cudaGraphExec_t>> graphs;
    uint32_t next_graph = 1;
    bool capturing = false;
    bool profiling_before_capture = false;
    // profiling
    bool profiling = false;
    std::vector<bvhgpu::ProfileRec> prof;
    std::vector<cudaEvent_t> event_pool;
    // launch configuration per kernel id (only the tunable kernels read theirs)
    bvhgpu_tune_config tune[BVHGPU_KERNEL_COUNT];
    bvhgpu_ctx() {
        // defaults: the configs the autotuner picked on GB300 for the displaced-icosphere frame
        // (single BLAS) and the instanced frame (two-level)
        for (auto& t : tune) t = bvhgpu_tune_config{128u, 5u, 256u, 16u, 8u, 2000u};
        tune[BVHGPU_K_TRACE_BLAS].refill = 1u;
        tune[BVHGPU_K_TRACE_SCENE].refill = 1u;
    }
};

// Frees every physics world of the context (physics.cu).
void bvhgpu_free_worlds(bvhgpu_ctx* ctx);

namespace bvhgpu {

// Launch bracket for per-kernel timing.
struct LaunchScope {
    bvhgpu_ctx* ctx;
    int kernel;
    cudaStream_t s;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    LaunchScope(bvhgpu_ctx* c, int k, cudaStream_t st);
    ~LaunchScope();
};

// ---- launchers (kernels_trace.cu) ------------------------------------------------------
cudaError_t launch_trace_blas(bvhgpu_ctx* ctx, const DeviceBlas& b, const float4* rays, uint32_t n, void* hits,
                              cudaStream_t s);
// `base`: index of the first ray in the caller's whole ray set (the bounce directions' random key is
// the ray's index there, so a ray set traced in parts gives the same bounces).
cudaError_t launch_bounce_plain(bvhgpu_ctx* ctx, const DeviceBlas& b, const float4* rays, uint32_t n, uint32_t seed,
                                void* hits0, void* hits1, cudaStream_t s, uint32_t base = 0);
// hit_count (may be null): primary hits are added to *hit_count.
cudaError_t launch_bounce_persistent(bvhgpu_ctx* ctx, const DeviceBlas& b, const float4* rays, uint32_t n,
                                     uint32_t seed, void* hits0, void* hits1, cudaStream_t s, uint32_t base = 0,
                                     uint32_t* hit_count = nullptr);
// The plain traversal with per-ray work counters summed into out[0..6] (TraceCounts order).
cudaError_t launch_trace_count(bvhgpu_ctx* ctx, const DeviceBlas& b, const float4* rays, uint32_t n, void* hits,
                               unsigned long long* out, cudaStream_t s);
// Adds the number of hit records with a primitive (prim != miss) among hits[0, n) to *count.
cudaError_t launch_count_hits(bvhgpu_ctx* ctx, const void* hits, uint32_t n, uint32_t* count, cudaStream_t s);
cudaError_t launch_bounce_rays(bvhgpu_ctx* ctx, const DeviceBlas& b, const float4* rays, const void* hits0,
                               uint32_t n, uint32_t seed, float4* out, uint8_t* valid, cudaStream_t s);
// True when the persistent batch's device table already describes `items` (no upload needed).
bool batch_table_current(const bvhgpu_ctx* ctx, const bvhgpu_batch_item* items, uint32_t nitems);
cudaError_t launch_trace_batch(bvhgpu_ctx* ctx, const std::vector<const DeviceBlas*>& blases,
                               const bvhgpu_batch_item* items, uint32_t nitems, const float4* rays, uint32_t nrays,
                               int mode, void* hits, cudaStream_t s);
cudaError_t launch_triangle_list(bvhgpu_ctx* ctx, const float* tris, uint32_t ntris, const float4* rays, uint32_t n,
                                 int mode, void* hits, cudaStream_t s);
cudaError_t launch_render_scene(bvhgpu_ctx* ctx, DeviceScene& sc, const bvhgpu_camera& cam, int w, int h, int acc,
                                const float* acc_params, int shader, const float* shader_params,
                                const ShadeEntry* d_shade, int lookup, uint8_t* d_rgba, cudaStream_t s);
cudaError_t launch_render(bvhgpu_ctx* ctx, const DeviceBlas& b, const bvhgpu_camera& cam, int w, int h, int acc,
                          const float* acc_params, int shader, const float* shader_params, const float* d_normals,
                          const float* d_tex_coords, const uint8_t* d_texels, uint32_t tex_w, uint32_t tex_h,
                          uint8_t* d_rgba, cudaStream_t s);

// ---- launchers (kernels_scene.cu) ------------------------------------------------------
cudaError_t launch_write_tris(bvhgpu_ctx* ctx, DeviceBlas& b, const float* d_tris9, cudaStream_t s);
// Rewrites the hidden trees' pairs, boxes and leaf bounds from b.tris; part of every triangle write.
cudaError_t launch_hidden_refresh(bvhgpu_ctx* ctx, DeviceBlas& b, cudaStream_t s);
cudaError_t launch_refit(bvhgpu_ctx* ctx, DeviceBlas& b, cudaStream_t s);
// Physics (physics.cu).
cudaError_t launch_world_start_frame(bvhgpu_ctx* ctx, DeviceWorld& w, cudaStream_t s);
cudaError_t launch_world_step(bvhgpu_ctx* ctx, DeviceWorld& w, float dt, cudaStream_t s);
cudaError_t launch_update_from_bodies(bvhgpu_ctx* ctx, DeviceScene& sc, const DeviceWorld& w, cudaStream_t s);
// BvhBuilder::build_for on the device (build_gpu.cu): mesh (host, n x 9 floats) is reordered in
// place, nodes_out (2n) and perm_out (optional) written; *what names a failure.
int build_bvh_device(bvhgpu_ctx* ctx, float* mesh, uint32_t n, bvhgpu_node* nodes_out, uint32_t* nodes_used,
                     uint32_t* perm_out, const char** what);
// Sets ctx->last_error to msg and returns code (the ABI's error path).
int record_error(bvhgpu_ctx* ctx, int code, const char* msg);
// A TLAS of n objects has 2n nodes and LeftRightIndex packs two 16-bit node indices (tlas.rs:18-22),
// so a scene holds at most 32,768 objects; the rebuild keeps its 40 B per object in shared memory
// up to kTlasSharedObjects objects and in the scene's global scratch above.
constexpr uint32_t kMaxSceneObjects = 32768;
constexpr uint32_t kTlasSharedObjects = 4096;
size_t tlas_smem_bytes(uint32_t nobj);  // the TLAS rebuild's per-object state
cudaError_t launch_tlas_rebuild(bvhgpu_ctx* ctx, DeviceScene& sc, cudaStream_t s);
cudaError_t launch_trace_scene(bvhgpu_ctx* ctx, DeviceScene& sc, const float4* rays, uint32_t n, void* hits,
                               cudaStream_t s);
cudaError_t launch_scene_bounce(bvhgpu_ctx* ctx, DeviceScene& sc, const float4* rays, uint32_t n, uint32_t seed,
                                void* hits0, void* hits1, cudaStream_t s);
cudaError_t launch_scene_bounce_rays(bvhgpu_ctx* ctx, DeviceScene& sc, const float4* rays, const void* hits0,
                                     uint32_t n, uint32_t seed, float4* out, uint8_t* valid, cudaStream_t s);
cudaError_t launch_wobble(bvhgpu_ctx* ctx, float* verts, const float* dirs, const float* r0, const float* phase,
                          uint32_t nv, float amp, float freq, const float* time, cudaStream_t s);
cudaError_t launch_animate_instances(bvhgpu_ctx* ctx, DeviceScene& sc, const float* rot0, const float* axis,
                                     const float* omega, const float* scale, const float* trans, const float* time,
                                     cudaStream_t s);
cudaError_t launch_advance_time(bvhgpu_ctx* ctx, float* time, float dt, cudaStream_t s);

// ---- launchers (kernels_adjoint.cu) ----------------------------------------------------
cudaError_t launch_mesh_update(bvhgpu_ctx* ctx, DeviceMesh& m, DeviceBlas& b, cudaStream_t s);
cudaError_t launch_lambert_forward(bvhgpu_ctx* ctx, DeviceMesh& m, const DeviceBlas& b, const float4* rays, uint32_t n,
                                   const float* light, float* image, void* hits, cudaStream_t s);
cudaError_t launch_mse_partials(bvhgpu_ctx* ctx, const float* image, const float* target, uint32_t n, double* partials,
                                cudaStream_t s);
cudaError_t launch_lambert_adjoint(bvhgpu_ctx* ctx, DeviceMesh& m, const float4* rays, uint32_t n, const float* light,
                                   const void* hits, const float* image, const float* target, float* grad,
                                   cudaStream_t s);
cudaError_t launch_sgd(bvhgpu_ctx* ctx, DeviceMesh& m, float* grad, float lr, cudaStream_t s);

// ---- host SAH build (host_build.cpp) ----------------------------------------------------
int build_bvh_host(bvhgpu_triangle* mesh, uint32_t n, bvhgpu_node* nodes_out, uint32_t* nodes_used,
                   uint32_t* perm_out);

}  // namespace bvhgpu
