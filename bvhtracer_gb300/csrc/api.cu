// C ABI of the bvhgpu library (include/bvhgpu.h): context, memory helpers, timing, BLAS and
// scene management, and the trace / refit / rebuild / render entry points.
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cfloat>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <type_traits>
#include <vector>

#include <unistd.h>

#include "common.cuh"
#include "internal.hpp"

namespace bvhgpu {

std::atomic<uint64_t> g_launches{0};

// NVTX range names per kernel id (BVHGPU_K_*): every launch is bracketed by a host range, so a timeline
// tool shows refit / TLAS rebuild / trace / render / adjoint phases.  Without a tool attached an NVTX
// call costs a branch.
static const char* const kRangeNames[BVHGPU_KERNEL_COUNT] = {
    "bvhgpu trace", "bvhgpu trace scene", "bvhgpu trace + bounce (persistent)", "bvhgpu bounce generation",
    "bvhgpu trace queue", "bvhgpu trace batch", "bvhgpu refit", "bvhgpu TLAS rebuild", "bvhgpu render",
    "bvhgpu other", "bvhgpu Lambert forward", "bvhgpu Lambert adjoint", "bvhgpu scene trace + bounce"};

LaunchScope::LaunchScope(bvhgpu_ctx* c, int k, cudaStream_t st) : ctx(c), kernel(k), s(st) {
    nvtxRangePushA(k >= 0 && k < BVHGPU_KERNEL_COUNT ? kRangeNames[k] : "bvhgpu");
    if (!ctx->profiling) return;
    if (ctx->event_pool.size() >= 2) {
        e1 = ctx->event_pool.back();
        ctx->event_pool.pop_back();
        e0 = ctx->event_pool.back();
        ctx->event_pool.pop_back();
    } else {
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
    }
    cudaEventRecord(e0, s);
}

LaunchScope::~LaunchScope() {
    nvtxRangePop();
    if (!e0) return;
    cudaEventRecord(e1, s);
    ctx->prof.push_back(ProfileRec{kernel, e0, e1});
}

}  // namespace bvhgpu

using namespace bvhgpu;

namespace {

static_assert(sizeof(bvhgpu_node) == 32, "bvhgpu_node layout");
static_assert(sizeof(bvhgpu_triangle) == 36, "bvhgpu_triangle layout");
static_assert(sizeof(bvhgpu_ray) == 32, "bvhgpu_ray layout");
static_assert(sizeof(bvhgpu_hit) == 20, "bvhgpu_hit layout");
static_assert(sizeof(bvhgpu_tlas_node) == 32, "bvhgpu_tlas_node layout");
static_assert(sizeof(bvhgpu_batch_item) == 16, "bvhgpu_batch_item layout");

int fail(bvhgpu_ctx* ctx, int code, const char* fmt, ...) {
    if (ctx) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        ctx->last_error = buf;
    }
    return code;
}

}  // namespace

int bvhgpu::record_error(bvhgpu_ctx* ctx, int code, const char* msg) { return fail(ctx, code, "%s", msg); }

namespace {

int cuda_fail(bvhgpu_ctx* ctx, cudaError_t e, const char* what) {
    return fail(ctx, BVHGPU_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(expr, what)                                    \
    do {                                                  \
        cudaError_t _e = (expr);                          \
        if (_e != cudaSuccess) return cuda_fail(ctx, _e, what); \
    } while (0)

cudaStream_t pick(bvhgpu_ctx* ctx, bvhgpu_stream s) { return s ? static_cast<cudaStream_t>(s) : ctx->stream; }

int ensure(bvhgpu_ctx* ctx, void** buf, size_t* cap, size_t need) {
    if (*cap >= need) return BVHGPU_OK;
    if (*buf) cudaFree(*buf);
    *buf = nullptr;
    *cap = 0;
    size_t want = std::max<size_t>(need, 1 << 20);
    cudaError_t e = cudaMalloc(buf, want);
    if (e != cudaSuccess) return fail(ctx, BVHGPU_ERR_OUT_OF_MEMORY, "cudaMalloc(%zu): %s", want, cudaGetErrorString(e));
    *cap = want;
    return BVHGPU_OK;
}

int read_errors(bvhgpu_ctx* ctx) {
    uint32_t flags = 0;
    CK(cudaMemcpy(&flags, ctx->d_err, sizeof(flags), cudaMemcpyDeviceToHost), "read error flags");
    if (flags) {
        CK(cudaMemset(ctx->d_err, 0, sizeof(uint32_t)), "reset error flags");
        if (flags & kErrStack) return fail(ctx, BVHGPU_ERR_STACK_DEPTH, "traversal stack overflow (tree too deep)");
        if (flags & kErrDeadline)
            return fail(ctx, BVHGPU_ERR_DEADLINE, "a launch stopped at the context's deadline; its outputs are incomplete");
        if (flags & kErrLookup)
            return fail(ctx, BVHGPU_ERR_INVALID_ARG,
                        "a hit's primitive index lies outside the looked-up model's shading data (the reference "
                        "indexes out of bounds and panics there)");
        return fail(ctx, BVHGPU_ERR_STEP_CAP, "traversal step cap exceeded (malformed tree)");
    }
    return BVHGPU_OK;
}

int finish(bvhgpu_ctx* ctx) {
    CK(cudaStreamSynchronize(ctx->stream), "stream synchronize");
    return read_errors(ctx);
}

DeviceBlas* find_blas(bvhgpu_ctx* ctx, uint32_t id) {
    auto it = ctx->blas.find(id);
    return it == ctx->blas.end() ? nullptr : &it->second;
}
DeviceScene* find_scene(bvhgpu_ctx* ctx, uint32_t id) {
    auto it = ctx->scenes.find(id);
    return it == ctx->scenes.end() ? nullptr : &it->second;
}

void free_blas(DeviceBlas& b) {
    cudaFree(b.nodes);
    cudaFree(b.tris);
    cudaFree(b.verts);
    cudaFree(b.pairs);
    cudaFree(b.parent);
    cudaFree(b.leaves);
    cudaFree(b.counters);
    cudaFree(b.tri_leaf);
    cudaFree(b.leaf_keys);
    cudaFree(b.hx);
    cudaFree(b.cones);
    cudaFree(b.hwork);
    cudaFree(b.hchunks);
    cudaFree(b.hchunk0);
    cudaFree(b.hpart);
    cudaFree(b.harrivals);
    cudaFree(b.normals);
    cudaFree(b.tex_coords);
    cudaFree(b.texels);
    b = DeviceBlas();
}

void free_mesh(DeviceMesh& m) {
    cudaFree(m.faces);
    cudaFree(m.verts);
    cudaFree(m.vnormals);
    cudaFree(m.sched);
    m = DeviceMesh();
}

DeviceMesh* find_mesh(bvhgpu_ctx* ctx, uint32_t id) {
    auto it = ctx->meshes.find(id);
    return it == ctx->meshes.end() ? nullptr : &it->second;
}

void free_scene(DeviceScene& s) {
    cudaFree(s.xf);
    cudaFree(s.inv);
    cudaFree(s.body_of);
    cudaFree(s.transform_init);
    cudaFree(s.obj_blas);
    cudaFree(s.blas_table);
    cudaFree(s.tlas);
    cudaFree(s.tlas_work);
    s = DeviceScene();
}

// Validates a reference node array and derives parent links, leaf list and depth.
int analyse_nodes(bvhgpu_ctx* ctx, const bvhgpu_node* nodes, uint32_t nodes_used, uint32_t ntris,
                  std::vector<uint32_t>& parent, std::vector<uint32_t>& leaves, uint32_t* depth,
                  std::vector<uint32_t>& tri_leaf) {
    parent.assign(nodes_used, 0xFFFFFFFFu);
    leaves.clear();
    std::vector<uint32_t> seen(nodes_used, 0);
    std::vector<std::pair<uint32_t, uint32_t>> st;
    st.push_back({0u, 1u});
    seen[0] = 1;
    uint32_t maxd = 0;
    uint64_t covered = 0;
    while (!st.empty()) {
        auto [i, d] = st.back();
        st.pop_back();
        maxd = std::max(maxd, d);
        const bvhgpu_node& n = nodes[i];
        if (n.primitive_count > 0) {
            if ((uint64_t)n.left_first + n.primitive_count > ntris)
                return fail(ctx, BVHGPU_ERR_INVALID_ARG, "leaf %u addresses triangles past %u", i, ntris);
            leaves.push_back(i);
            covered += n.primitive_count;
        } else {
            uint32_t l = n.left_first;
            if (l < 2 || (uint64_t)l + 1 >= nodes_used || l <= i)
                return fail(ctx, BVHGPU_ERR_INVALID_ARG, "branch %u has bad child index %u", i, l);
            if (seen[l] || seen[l + 1]) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "node %u reached twice", l);
            seen[l] = seen[l + 1] = 1;
            parent[l] = i;
            parent[l + 1] = i;
            st.push_back({l, d + 1});
            st.push_back({l + 1, d + 1});
        }
    }
    (void)covered;
    *depth = maxd;
    tri_leaf.assign(ntris, 0xFFFFFFFFu);
    for (uint32_t li = 0; li < leaves.size(); ++li) {
        const bvhgpu_node& n = nodes[leaves[li]];
        for (uint32_t t = n.left_first; t < n.left_first + n.primitive_count; ++t) {
            if (tri_leaf[t] != 0xFFFFFFFFu)
                return fail(ctx, BVHGPU_ERR_INVALID_ARG, "triangle %u belongs to two leaves", t);
            tri_leaf[t] = li;
        }
    }
    return BVHGPU_OK;
}

void pack_nodes(const bvhgpu_node* nodes, uint32_t n, std::vector<float>& out) {
    out.resize(8ull * n);
    for (uint32_t i = 0; i < n; ++i) {
        float* o = &out[8ull * i];
        o[0] = nodes[i].bounds_min[0];
        o[1] = nodes[i].bounds_min[1];
        o[2] = nodes[i].bounds_min[2];
        std::memcpy(&o[3], &nodes[i].left_first, 4);
        o[4] = nodes[i].bounds_max[0];
        o[5] = nodes[i].bounds_max[1];
        o[6] = nodes[i].bounds_max[2];
        std::memcpy(&o[7], &nodes[i].primitive_count, 4);
    }
}

// Hidden trees over the leaves with at least kHiddenMinLeaf triangles, built by binned SAH: a range
// of triangles is split at the cheapest of 15 planes (16 bins of the centroids along the widest
// centroid axis, cost = area x count of each side), in halves by index order when the centroids
// coincide or below 32 binary levels, down to at most kHiddenLeafTris triangles stored as packed
// pairs (a padding slot is all zero with index 0xFFFFFFFF).  Two levels of splits make one 4-wide
// node.  Hidden nodes get indices from nodes_used on, a node's children consecutive, allocated
// depth first; the boxes and the leaf bounds Q, B and normal cone are written
// by the refresh kernels from `work`.  Only speed depends on the tree's shape.
struct HiddenPlan {
    std::vector<float> nodes;  // 8 floats per hidden node (boxes 0 until refreshed)
    std::vector<uint2> table;  // per triangle index, rounded up to even (empty: no hidden tree)
    std::vector<uint2> slots;  // per hidden pair
    std::vector<uint4> work;   // per hidden node (box), then per cone
    std::vector<uint2> chunks;    // {group, first pair}: each group in kRefreshChunk-pair chunks
    std::vector<uint32_t> chunk0;  // first chunk of each group, then the total
    uint32_t nbox_chunks = 0;      // chunks of the node groups (they come first)
    uint32_t nhid = 0, nhp = 0, ncones = 0, depth = 0;
};

struct SahTri {
    float c[3], lo[3], hi[3];
};

inline float half_area(const float lo[3], const float hi[3]) {
    const float e0 = hi[0] - lo[0], e1 = hi[1] - lo[1], e2 = hi[2] - lo[2];
    return e0 * e1 + e1 * e2 + e2 * e0;
}

// Reorders ids[a, b) into two non-empty parts by the binned SAH; returns the split position.
uint32_t sah_split(std::vector<uint32_t>& ids, const std::vector<SahTri>& info, uint32_t a, uint32_t b) {
    const uint32_t mid = a + (b - a) / 2;
    float cl[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, ch[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (uint32_t j = a; j < b; ++j)
        for (int k = 0; k < 3; ++k) {
            cl[k] = std::min(cl[k], info[ids[j]].c[k]);
            ch[k] = std::max(ch[k], info[ids[j]].c[k]);
        }
    int ax = 0;
    for (int k = 1; k < 3; ++k)
        if (ch[k] - cl[k] > ch[ax] - cl[ax]) ax = k;
    const float ext = ch[ax] - cl[ax];
    if (!(ext > 0.0f) || !(ext < FLT_MAX)) return mid;
    constexpr int kBins = 16;
    auto bin_of = [&](uint32_t id) {
        const float x = (info[id].c[ax] - cl[ax]) / ext * (float)kBins;
        return x >= 0.0f ? std::min(kBins - 1, (int)x) : 0;  // NaN -> 0
    };
    uint32_t cnt[kBins] = {};
    float blo[kBins][3], bhi[kBins][3];
    for (int i = 0; i < kBins; ++i)
        for (int k = 0; k < 3; ++k) {
            blo[i][k] = FLT_MAX;
            bhi[i][k] = -FLT_MAX;
        }
    for (uint32_t j = a; j < b; ++j) {
        const int i = bin_of(ids[j]);
        ++cnt[i];
        for (int k = 0; k < 3; ++k) {
            blo[i][k] = std::min(blo[i][k], info[ids[j]].lo[k]);
            bhi[i][k] = std::max(bhi[i][k], info[ids[j]].hi[k]);
        }
    }
    float right_cost[kBins] = {};
    float rlo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, rhi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    uint32_t rn = 0;
    for (int i = kBins - 1; i > 0; --i) {  // right side = bins i..15
        rn += cnt[i];
        for (int k = 0; k < 3; ++k) {
            rlo[k] = std::min(rlo[k], blo[i][k]);
            rhi[k] = std::max(rhi[k], bhi[i][k]);
        }
        right_cost[i] = rn ? half_area(rlo, rhi) * (float)rn : 0.0f;
    }
    float llo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, lhi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    uint32_t ln = 0;
    float best = FLT_MAX;
    int best_bin = -1;  // left side = bins 0..best_bin
    for (int i = 0; i < kBins - 1; ++i) {
        ln += cnt[i];
        for (int k = 0; k < 3; ++k) {
            llo[k] = std::min(llo[k], blo[i][k]);
            lhi[k] = std::max(lhi[k], bhi[i][k]);
        }
        if (ln == 0 || ln == b - a) continue;
        const float cost = half_area(llo, lhi) * (float)ln + right_cost[i + 1];
        if (cost < best) {
            best = cost;
            best_bin = i;
        }
    }
    if (best_bin < 0) return mid;
    auto it = std::stable_partition(ids.begin() + a, ids.begin() + b,
                                    [&](uint32_t id) { return bin_of(id) <= best_bin; });
    return (uint32_t)(it - ids.begin());
}

void plan_hidden(const bvhgpu_node* nodes, uint32_t nodes_used, const std::vector<uint32_t>& leaves,
                 const bvhgpu_triangle* tris, uint32_t ntris, HiddenPlan& hp) {
    const uint32_t P0 = pairs_in_order(ntris);
    std::vector<uint32_t> ids;
    std::vector<SahTri> info;
    std::vector<uint4> cones;  // cone work: {first pair, end pair, ~0, cone}
    // (first, count) of the subtree over ids[a, b) at `depth` (4-wide levels) below the hidden
    // root; its pairs are allocated contiguously.  An interior node gets its children from two
    // levels of binary SAH splits (2 to 4 ranges); nodes below the root get their own cone.
    auto make = [&](auto&& self, uint32_t a, uint32_t b, uint32_t depth, uint32_t gov) -> uint2 {
        hp.depth = std::max(hp.depth, depth);
        if (b - a <= kHiddenLeafTris) {
            const uint32_t np = (b - a + 1) / 2;
            const uint32_t p0 = P0 + hp.nhp;
            for (uint32_t q = 0; q < np; ++q) {
                const uint32_t s0 = a + 2 * q;
                hp.slots.push_back(make_uint2(ids[s0], s0 + 1 < b ? ids[s0 + 1] : kMiss));
            }
            hp.nhp += np;
            return make_uint2(p0, kHiddenLeaf | np);
        }
        const uint32_t pa = P0 + hp.nhp;
        const uint32_t own = depth >= 1 ? hp.ncones++ : kNoRefresh;
        if (own != kNoRefresh) gov = own;
        // SAH down to 32 binary levels, then halves (a balanced rest keeps the stack need bounded)
        auto split = [&](uint32_t x, uint32_t y) {
            return 2 * depth < 32 ? sah_split(ids, info, x, y) : x + (y - x) / 2;
        };
        uint32_t ranges[5];
        uint32_t nr = 0;
        const uint32_t m = split(a, b);
        ranges[nr++] = a;
        if (m - a > kHiddenLeafTris) ranges[nr++] = split(a, m);
        ranges[nr++] = m;
        if (b - m > kHiddenLeafTris) ranges[nr++] = split(m, b);
        ranges[nr] = b;
        const uint32_t k = nr;  // 2..4 children
        const uint32_t li = hp.nhid;
        hp.nhid += k;
        hp.nodes.resize(8ull * hp.nhid, 0.0f);
        hp.work.resize(hp.nhid);
        for (uint32_t c = 0; c < k; ++c) {
            const uint32_t pc = P0 + hp.nhp;
            const uint2 meta = self(self, ranges[c], ranges[c + 1], depth + 1, gov);
            float* o = &hp.nodes[8ull * (li + c)];
            std::memcpy(&o[3], &meta.x, 4);
            std::memcpy(&o[7], &meta.y, 4);
            hp.work[li + c] = make_uint4(pc, P0 + hp.nhp, nodes_used + li + c, kNoRefresh);
        }
        if (own != kNoRefresh) cones.push_back(make_uint4(pa, P0 + hp.nhp, kNoRefresh, own));
        return make_uint2(nodes_used + li, kHiddenInterior | ((k - 1) << kWideShift) | gov);
    };
    info.resize(ntris);
    for (uint32_t li : leaves) {
        const bvhgpu_node& n = nodes[li];
        if (n.primitive_count < kHiddenMinLeaf) continue;
        if (hp.table.empty()) hp.table.assign(hidden_table_u2(ntris), make_uint2(0u, 0u));
        ids.resize(n.primitive_count);
        for (uint32_t k = 0; k < n.primitive_count; ++k) {
            const uint32_t t = n.left_first + k;
            const float* v = tris[t].vertices;
            SahTri& s = info[t];
            for (int a = 0; a < 3; ++a) {
                s.c[a] = (v[a] + v[3 + a] + v[6 + a]) / 3.0f;
                s.lo[a] = std::min(v[a], std::min(v[3 + a], v[6 + a]));
                s.hi[a] = std::max(v[a], std::max(v[3 + a], v[6 + a]));
            }
            ids[k] = t;
        }
        const uint32_t pa = P0 + hp.nhp;
        const uint32_t root_cone = hp.ncones++;
        const uint2 root = make(make, 0, n.primitive_count, 0, root_cone);  // interior: >= 16 triangles
        hp.table[n.left_first] = root;
        cones.push_back(make_uint4(pa, P0 + hp.nhp, kNoRefresh, root_cone));
    }
    hp.work.insert(hp.work.end(), cones.begin(), cones.end());
    for (uint32_t j = 0; j < hp.work.size(); ++j) {
        hp.chunk0.push_back((uint32_t)hp.chunks.size());
        for (uint32_t p = hp.work[j].x; p < hp.work[j].y; p += kRefreshChunk) hp.chunks.push_back(make_uint2(j, p));
        if (hp.work[j].z != kNoRefresh) hp.nbox_chunks = (uint32_t)hp.chunks.size();  // node groups come first
    }
    hp.chunk0.push_back((uint32_t)hp.chunks.size());
}

}  // namespace

extern "C" {

int bvhgpu_create(bvhgpu_ctx** out, int device) {
    if (!out) return BVHGPU_ERR_INVALID_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return BVHGPU_ERR_NO_DEVICE;
    if (device < 0 || device >= ndev) return BVHGPU_ERR_INVALID_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return BVHGPU_ERR_CUDA;
    bvhgpu_ctx* ctx = new bvhgpu_ctx();
    ctx->device = device;
    cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    cudaDeviceGetAttribute(&ctx->pageable_access, cudaDevAttrPageableMemoryAccess, device);
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&ctx->d_err, 4 * sizeof(uint32_t)) != cudaSuccess ||  // flags, pad, deadline (u64 ns)
        cudaMalloc(&ctx->d_scratch, 64 * sizeof(uint32_t)) != cudaSuccess ||
        cudaMallocHost(&ctx->host_word, 64) != cudaSuccess) {
        delete ctx;
        return BVHGPU_ERR_CUDA;
    }
    cudaMemset(ctx->d_err, 0, 4 * sizeof(uint32_t));
    cudaMemset(ctx->d_scratch, 0, 64 * sizeof(uint32_t));
    cudaDeviceSynchronize();
    *out = ctx;
    return BVHGPU_OK;
}

int bvhgpu_destroy(bvhgpu_ctx* ctx) {
    if (!ctx) return BVHGPU_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (auto& kv : ctx->blas) free_blas(kv.second);
    for (auto& kv : ctx->scenes) free_scene(kv.second);
    for (auto& kv : ctx->meshes) free_mesh(kv.second);
    bvhgpu_free_worlds(ctx);
    for (auto& kv : ctx->graphs) {
        cudaGraphExecDestroy(kv.second.second);
        cudaGraphDestroy(kv.second.first);
    }
    cudaFree(ctx->mse_partials);
    for (auto& r : ctx->prof) {
        cudaEventDestroy(r.start);
        cudaEventDestroy(r.stop);
    }
    for (auto e : ctx->event_pool) cudaEventDestroy(e);
    cudaFree(ctx->d_err);
    cudaFree(ctx->d_scratch);
    cudaFree(ctx->l2_flush);
    cudaFree(ctx->stage_in);
    cudaFree(ctx->stage_out);
    cudaFree(ctx->stage_out2);
    cudaFree(ctx->bounce_rays);
    cudaFree(ctx->bounce_pix);
    cudaFree(ctx->batch_table);
    cudaFreeHost(ctx->host_word);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return BVHGPU_OK;
}

const char* bvhgpu_last_error(const bvhgpu_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

uint64_t bvhgpu_launch_count(void) { return g_launches.load(); }

int bvhgpu_sync(bvhgpu_ctx* ctx) {
    if (!ctx) return BVHGPU_ERR_INVALID_ARG;
    return finish(ctx);
}

bvhgpu_stream bvhgpu_get_stream(bvhgpu_ctx* ctx) { return ctx ? ctx->stream : nullptr; }

// ---- memory helpers -------------------------------------------------------------------------

int bvhgpu_device_alloc(bvhgpu_ctx* ctx, size_t bytes, void** out) {
    if (!ctx || !out) return BVHGPU_ERR_INVALID_ARG;
    cudaError_t e = cudaMalloc(out, std::max<size_t>(bytes, 16));
    if (e != cudaSuccess) return fail(ctx, BVHGPU_ERR_OUT_OF_MEMORY, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
    return BVHGPU_OK;
}
int bvhgpu_device_free(bvhgpu_ctx* ctx, void* p) {
    if (!ctx) return BVHGPU_ERR_INVALID_ARG;
    CK(cudaFree(p), "cudaFree");
    return BVHGPU_OK;
}
int bvhgpu_host_alloc(bvhgpu_ctx* ctx, size_t bytes, void** out) {
    if (!ctx || !out) return BVHGPU_ERR_INVALID_ARG;
    cudaError_t e = cudaMallocHost(out, std::max<size_t>(bytes, 16));
    if (e != cudaSuccess) return fail(ctx, BVHGPU_ERR_OUT_OF_MEMORY, "cudaMallocHost(%zu): %s", bytes, cudaGetErrorString(e));
    return BVHGPU_OK;
}
int bvhgpu_host_free(bvhgpu_ctx* ctx, void* p) {
    if (!ctx) return BVHGPU_ERR_INVALID_ARG;
    CK(cudaFreeHost(p), "cudaFreeHost");
    return BVHGPU_OK;
}
int bvhgpu_copy_to_device(bvhgpu_ctx* ctx, void* dst, const void* src, size_t bytes, bvhgpu_stream s) {
    if (!ctx || (bytes && (!dst || !src))) return BVHGPU_ERR_INVALID_ARG;
    CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, pick(ctx, s)), "copy to device");
    return BVHGPU_OK;
}
int bvhgpu_copy_to_host(bvhgpu_ctx* ctx, void* dst, const void* src, size_t bytes, bvhgpu_stream s) {
    if (!ctx || (bytes && (!dst || !src))) return BVHGPU_ERR_INVALID_ARG;
    CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, pick(ctx, s)), "copy to host");
    return BVHGPU_OK;
}
int bvhgpu_memset_device(bvhgpu_ctx* ctx, void* dst, int value, size_t bytes, bvhgpu_stream s) {
    if (!ctx || (bytes && !dst)) return BVHGPU_ERR_INVALID_ARG;
    CK(cudaMemsetAsync(dst, value, bytes, pick(ctx, s)), "memset");
    return BVHGPU_OK;
}
int bvhgpu_flush_l2(bvhgpu_ctx* ctx, bvhgpu_stream s) {
    if (!ctx) return BVHGPU_ERR_INVALID_ARG;
    if (!ctx->l2_flush) {
        int l2 = 0;
        cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, ctx->device);
        ctx->l2_flush_bytes = std::max<size_t>((size_t)l2 * 2, 256ull << 20);
        CK(cudaMalloc(&ctx->l2_flush, ctx->l2_flush_bytes), "alloc L2 flush buffer");
    }
    static int flip = 0;
    flip ^= 1;
    CK(cudaMemsetAsync(ctx->l2_flush, flip, ctx->l2_flush_bytes, pick(ctx, s)), "L2 flush");
    return BVHGPU_OK;
}

// ---- timing -------------------------------------------------------------------------------------

int bvhgpu_event_create(bvhgpu_ctx* ctx, void** ev) {
    if (!ctx || !ev) return BVHGPU_ERR_INVALID_ARG;
    cudaEvent_t e;
    CK(cudaEventCreate(&e), "event create");
    *ev = e;
    return BVHGPU_OK;
}
int bvhgpu_event_destroy(bvhgpu_ctx* ctx, void* ev) {
    if (!ctx || !ev) return BVHGPU_ERR_INVALID_ARG;
    CK(cudaEventDestroy(static_cast<cudaEvent_t>(ev)), "event destroy");
    return BVHGPU_OK;
}
int bvhgpu_event_record(bvhgpu_ctx* ctx, void* ev, bvhgpu_stream s) {
    if (!ctx || !ev) return BVHGPU_ERR_INVALID_ARG;
    CK(cudaEventRecord(static_cast<cudaEvent_t>(ev), pick(ctx, s)), "event record");
    return BVHGPU_OK;
}
int bvhgpu_event_elapsed_ms(bvhgpu_ctx* ctx, void* start, void* stop, float* ms) {
    if (!ctx || !start || !stop || !ms) return BVHGPU_ERR_INVALID_ARG;
    CK(cudaEventSynchronize(static_cast<cudaEvent_t>(stop)), "event synchronize");
    CK(cudaEventElapsedTime(ms, static_cast<cudaEvent_t>(start), static_cast<cudaEvent_t>(stop)), "event elapsed");
    return BVHGPU_OK;
}
int bvhgpu_profile_enable(bvhgpu_ctx* ctx, int enable) {
    if (!ctx) return BVHGPU_ERR_INVALID_ARG;
    ctx->profiling = enable != 0;
    return BVHGPU_OK;
}
int bvhgpu_profile_read(bvhgpu_ctx* ctx, double* ms, uint64_t* launches) {
    if (!ctx) return BVHGPU_ERR_INVALID_ARG;
    for (int k = 0; k < BVHGPU_KERNEL_COUNT; ++k) {
        if (ms) ms[k] = 0.0;
        if (launches) launches[k] = 0;
    }
    for (auto& r : ctx->prof) {
        CK(cudaEventSynchronize(r.stop), "event synchronize");
        float t = 0.0f;
        CK(cudaEventElapsedTime(&t, r.start, r.stop), "event elapsed");
        if (ms) ms[r.kernel] += t;
        if (launches) launches[r.kernel] += 1;
        ctx->event_pool.push_back(r.start);
        ctx->event_pool.push_back(r.stop);
    }
    ctx->prof.clear();
    return BVHGPU_OK;
}

// ---- BLAS -------------------------------------------------------------------------------------

int bvhgpu_build_bvh_host(bvhgpu_triangle* mesh, uint32_t n, bvhgpu_node* nodes_out, uint32_t* nodes_used) {
    return build_bvh_host(mesh, n, nodes_out, nodes_used, nullptr);
}

int bvhgpu_build_bvh_host_indexed(bvhgpu_triangle* mesh, uint32_t n, bvhgpu_node* nodes_out, uint32_t* nodes_used,
                                  uint32_t* perm_out) {
    if (!perm_out) return BVHGPU_ERR_INVALID_ARG;
    return build_bvh_host(mesh, n, nodes_out, nodes_used, perm_out);
}

int bvhgpu_blas_upload(bvhgpu_ctx* ctx, const bvhgpu_node* nodes, uint32_t nodes_used, const bvhgpu_triangle* tris,
                       uint32_t ntris, uint32_t* blas_id) {
    if (!ctx || !nodes || !tris || !blas_id || nodes_used < 1 || ntris == 0)
        return fail(ctx, BVHGPU_ERR_INVALID_ARG, "blas_upload: null pointer or empty mesh");
    std::vector<uint32_t> parent, leaves, tri_leaf;
    uint32_t depth = 0;
    int rc = analyse_nodes(ctx, nodes, nodes_used, ntris, parent, leaves, &depth, tri_leaf);
    if (rc) return rc;
    DeviceBlas b;
    b.nodes_used = nodes_used;
    b.ntris = ntris;
    b.nleaves = (uint32_t)leaves.size();
    b.root_count = nodes[0].primitive_count;
    b.root_first = nodes[0].left_first;
    std::vector<float> packed;
    pack_nodes(nodes, nodes_used, packed);
    // refit keys start at the identities: min keys all-ones, max keys zero (6 per leaf)
    std::vector<unsigned long long> key_init(6 * std::max<size_t>(1, leaves.size()), 0ull);
    for (size_t li = 0; li < key_init.size() / 6; ++li)
        for (int k = 0; k < 3; ++k) key_init[6 * li + k] = 0xFFFFFFFFFFFFFFFFull;
    HiddenPlan hp;
    plan_hidden(nodes, nodes_used, leaves, tris, ntris, hp);
    b.nhid = hp.nhid;
    b.nhp = hp.nhp;
    b.ncones = hp.ncones;
    b.nwork = (uint32_t)hp.work.size();
    b.nchunks = (uint32_t)hp.chunks.size();
    b.nbox_chunks = hp.nbox_chunks;
    const size_t part_bytes = std::max(sizeof(float2), sizeof(RefreshAgg)) * std::max<size_t>(1, hp.chunks.size());
    b.ref_depth = depth;
    b.depth = depth + 3 * hp.depth;  // a 4-wide hidden level can leave 3 children pending
    const uint64_t nodes_all = (uint64_t)nodes_used + hp.nhid + 1;  // + a spare record (4-wide reads)
    const uint64_t pairs_all = (uint64_t)pairs_in_order(ntris) + hp.nhp;
    const uint64_t hx_bytes = hp.table.empty() ? 0 : 8ull * hidden_table_u2(ntris) + 8ull * std::max<uint32_t>(1, hp.nhp);
    void* d_tris9 = nullptr;
    cudaError_t e = cudaSuccess;
    auto cleanup = [&]() {
        cudaFree(d_tris9);
        free_blas(b);
    };
    if ((e = cudaMalloc(&b.nodes, 32ull * nodes_all)) != cudaSuccess ||
        (e = cudaMalloc(&b.tris, 48ull * ntris)) != cudaSuccess ||
        (e = cudaMalloc(&b.verts, 48ull * ntris)) != cudaSuccess ||
        (e = cudaMalloc(&b.pairs, 80ull * pairs_all)) != cudaSuccess ||
        (e = cudaMalloc(&b.parent, 4ull * nodes_used)) != cudaSuccess ||
        (e = cudaMalloc(&b.leaves, 4ull * std::max<size_t>(1, leaves.size()))) != cudaSuccess ||
        (e = cudaMalloc(&b.counters, 4ull * nodes_used)) != cudaSuccess ||
        (e = cudaMalloc(&b.tri_leaf, 4ull * ntris)) != cudaSuccess ||
        (e = cudaMalloc(&b.leaf_keys, 48ull * std::max<size_t>(1, leaves.size()))) != cudaSuccess ||
        (e = cudaMalloc(&d_tris9, 36ull * ntris)) != cudaSuccess ||
        (hx_bytes && (e = cudaMalloc(&b.hx, hx_bytes)) != cudaSuccess) ||
        (b.ncones && (e = cudaMalloc(&b.cones, 32ull * b.ncones)) != cudaSuccess) ||
        (b.nwork && (e = cudaMalloc(&b.hwork, 16ull * b.nwork)) != cudaSuccess) ||
        (b.nwork && (e = cudaMalloc(&b.hchunks, 8ull * b.nchunks)) != cudaSuccess) ||
        (b.nwork && (e = cudaMalloc(&b.hchunk0, 4ull * (b.nwork + 1))) != cudaSuccess) ||
        (b.nwork && (e = cudaMalloc(&b.hpart, part_bytes)) != cudaSuccess) ||
        (b.nwork && (e = cudaMalloc(&b.harrivals, 4ull * b.nwork)) != cudaSuccess)) {
        cleanup();
        return fail(ctx, BVHGPU_ERR_OUT_OF_MEMORY, "blas_upload: %s", cudaGetErrorString(e));
    }
    if ((e = cudaMemcpy(b.nodes, packed.data(), 32ull * nodes_used, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(b.parent, parent.data(), 4ull * nodes_used, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(b.leaves, leaves.data(), 4ull * leaves.size(), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemset(b.counters, 0, 4ull * nodes_used)) != cudaSuccess ||
        (e = cudaMemset(b.nodes + 2ull * (nodes_all - 1), 0, 32)) != cudaSuccess ||
        (e = cudaMemcpy(b.tri_leaf, tri_leaf.data(), 4ull * ntris, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(b.leaf_keys, key_init.data(), 8ull * key_init.size(), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemset(b.pairs, 0, 80ull * pairs_all)) != cudaSuccess ||
        (e = cudaMemcpy(d_tris9, tris, 36ull * ntris, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (hp.nhid && (e = cudaMemcpy(b.nodes + 2ull * nodes_used, hp.nodes.data(), 32ull * hp.nhid,
                                    cudaMemcpyHostToDevice)) != cudaSuccess) ||
        (hx_bytes && (e = cudaMemcpy(b.hx, hp.table.data(), 8ull * hp.table.size(), cudaMemcpyHostToDevice)) != cudaSuccess) ||
        (hx_bytes && hp.nhp &&
         (e = cudaMemcpy(b.hx + hp.table.size(), hp.slots.data(), 8ull * hp.nhp, cudaMemcpyHostToDevice)) != cudaSuccess) ||
        (b.nwork && (e = cudaMemcpy(b.hwork, hp.work.data(), 16ull * b.nwork, cudaMemcpyHostToDevice)) != cudaSuccess) ||
        (b.nwork && (e = cudaMemcpy(b.hchunks, hp.chunks.data(), 8ull * b.nchunks, cudaMemcpyHostToDevice)) != cudaSuccess) ||
        (b.nwork && (e = cudaMemcpy(b.hchunk0, hp.chunk0.data(), 4ull * (b.nwork + 1), cudaMemcpyHostToDevice)) != cudaSuccess) ||
        (b.nwork && (e = cudaMemset(b.harrivals, 0, 4ull * b.nwork)) != cudaSuccess) ||
        (e = launch_write_tris(ctx, b, static_cast<const float*>(d_tris9), ctx->stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess) {
        cleanup();
        return cuda_fail(ctx, e, "blas_upload");
    }
    cudaFree(d_tris9);
    uint32_t id = ctx->next_blas++;
    ctx->blas[id] = b;
    *blas_id = id;
    return BVHGPU_OK;
}

int bvhgpu_blas_free(bvhgpu_ctx* ctx, uint32_t blas_id) {
    if (!ctx) return BVHGPU_ERR_INVALID_ARG;
    DeviceBlas* b = find_blas(ctx, blas_id);
    if (!b) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown BLAS %u", blas_id);
    cudaStreamSynchronize(ctx->stream);
    free_blas(*b);
    ctx->blas.erase(blas_id);
    return BVHGPU_OK;
}

int bvhgpu_blas_info(bvhgpu_ctx* ctx, uint32_t blas_id, uint32_t* nodes_used, uint32_t* ntris, uint32_t* depth) {
    if (!ctx) return BVHGPU_ERR_INVALID_ARG;
    DeviceBlas* b = find_blas(ctx, blas_id);
    if (!b) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown BLAS %u", blas_id);
    if (nodes_used) *nodes_used = b->nodes_used;
    if (ntris) *ntris = b->ntris;
    if (depth) *depth = b->ref_depth;
    return BVHGPU_OK;
}

int bvhgpu_blas_hidden(bvhgpu_ctx* ctx, uint32_t blas_id, uint32_t* nodes, uint32_t* pairs, uint32_t* depth) {
    if (!ctx) return BVHGPU_ERR_INVALID_ARG;
    DeviceBlas* b = find_blas(ctx, blas_id);
    if (!b) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown BLAS %u", blas_id);
    if (nodes) *nodes = b->nhid;
    if (pairs) *pairs = b->nhp;
    if (depth) *depth = (b->depth - b->ref_depth) / 3;
    return BVHGPU_OK;
}

int bvhgpu_set_deadline(bvhgpu_ctx* ctx, uint64_t ns) {
    if (!ctx) return BVHGPU_ERR_INVALID_ARG;
    if (ctx->capturing) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "set_deadline: not allowed during capture");
    CK(cudaMemcpyAsync(ctx->d_err + 2, &ns, sizeof(ns), cudaMemcpyHostToDevice, ctx->stream), "deadline");
    CK(cudaStreamSynchronize(ctx->stream), "stream synchronize");
    return BVHGPU_OK;
}

int bvhgpu_blas_hidden_download(bvhgpu_ctx* ctx, uint32_t blas_id, float* nodes, float* cones, uint32_t* slots,
                                uint32_t* table, uint32_t* ncones) {
    if (!ctx) return BVHGPU_ERR_INVALID_ARG;
    if (ctx->capturing) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "hidden_download: not allowed during capture");
    DeviceBlas* b = find_blas(ctx, blas_id);
    if (!b) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown BLAS %u", blas_id);
    if (ncones) *ncones = b->ncones;
    CK(cudaStreamSynchronize(ctx->stream), "stream synchronize");
    if (nodes && b->nhid)
        CK(cudaMemcpy(nodes, b->nodes + 2ull * b->nodes_used, 32ull * b->nhid, cudaMemcpyDeviceToHost), "hidden nodes");
    if (cones && b->ncones) CK(cudaMemcpy(cones, b->cones, 32ull * b->ncones, cudaMemcpyDeviceToHost), "cones");
    if (b->hx != nullptr) {
        const size_t t = hidden_table_u2(b->ntris);
        if (slots && b->nhp) CK(cudaMemcpy(slots, b->hx + t, 8ull * b->nhp, cudaMemcpyDeviceToHost), "pair slots");
        if (table) CK(cudaMemcpy(table, b->hx, 8ull * t, cudaMemcpyDeviceToHost), "hidden table");
    } else if (table) {
        std::memset(table, 0, 8ull * hidden_table_u2(b->ntris));
    }
    return BVHGPU_OK;
}

// The kernels read a ray as two float4 and write a hit record field by field, so a ray array the
// GPU reads in place must be 16-byte aligned and a hit array 4-byte aligned (cudaMalloc,
// bvhgpu_device_alloc and bvhgpu_host_alloc memory is; a view at an odd offset need not be).
static bool rays_aligned(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }
static bool hits_aligned(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 3u) == 0; }
static int misaligned(bvhgpu_ctx* ctx, const char* fn) {
    return fail(ctx, BVHGPU_ERR_INVALID_ARG, "%s: ray arrays must be 16-byte and hit arrays 4-byte aligned", fn);
}

int bvhgpu_blas_trace_counts(bvhgpu_ctx* ctx, uint32_t blas_id, const bvhgpu_ray* d_rays, uint32_t n,
                             bvhgpu_hit* d_hits, uint64_t counts[7]) {
    if (!ctx || !counts || (n && (!d_rays || !d_hits))) return BVHGPU_ERR_INVALID_ARG;
    if (n && (!rays_aligned(d_rays) || !hits_aligned(d_hits))) return misaligned(ctx, "trace_counts");
    if (ctx->capturing) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "trace_counts: not allowed during capture");
    DeviceBlas* b = find_blas(ctx, blas_id);
    if (!b) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown BLAS %u", blas_id);
    unsigned long long* d_out = reinterpret_cast<unsigned long long*>(ctx->d_scratch + 32);  // 7 x u64
    CK(cudaMemsetAsync(d_out, 0, 7 * sizeof(unsigned long long), ctx->stream), "counters");
    CK(launch_trace_count(ctx, *b, reinterpret_cast<const float4*>(d_rays), n, d_hits, d_out, ctx->stream),
       "trace (counting)");
    unsigned long long h[7];
    CK(cudaMemcpyAsync(h, d_out, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream), "counters");
    const int rc = finish(ctx);
    if (rc) return rc;
    for (int k = 0; k < 7; ++k) counts[k] = h[k];
    return BVHGPU_OK;
}

int bvhgpu_blas_update_vertices_async(bvhgpu_ctx* ctx, uint32_t blas_id, const bvhgpu_triangle* d_tris,
                                      bvhgpu_stream s) {
    if (!ctx || !d_tris) return BVHGPU_ERR_INVALID_ARG;
    DeviceBlas* b = find_blas(ctx, blas_id);
    if (!b) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown BLAS %u", blas_id);
    CK(launch_write_tris(ctx, *b, reinterpret_cast<const float*>(d_tris), pick(ctx, s)), "write triangles");
    return BVHGPU_OK;
}

int bvhgpu_blas_update_vertices(bvhgpu_ctx* ctx, uint32_t blas_id, const bvhgpu_triangle* tris) {
    if (!ctx || !tris) return BVHGPU_ERR_INVALID_ARG;
    DeviceBlas* b = find_blas(ctx, blas_id);
    if (!b) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown BLAS %u", blas_id);
    int rc = ensure(ctx, &ctx->stage_in, &ctx->stage_in_bytes, 36ull * b->ntris);
    if (rc) return rc;
    CK(cudaMemcpyAsync(ctx->stage_in, tris, 36ull * b->ntris, cudaMemcpyHostToDevice, ctx->stream), "upload vertices");
    CK(launch_write_tris(ctx, *b, static_cast<const float*>(ctx->stage_in), ctx->stream), "write triangles");
    return finish(ctx);
}

int bvhgpu_blas_refit_async(bvhgpu_ctx* ctx, uint32_t blas_id, bvhgpu_stream s) {
    if (!ctx) return BVHGPU_ERR_INVALID_ARG;
    DeviceBlas* b = find_blas(ctx, blas_id);
    if (!b) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown BLAS %u", blas_id);
    CK(launch_refit(ctx, *b, pick(ctx, s)), "refit");
    return BVHGPU_OK;
}

int bvhgpu_blas_refit(bvhgpu_ctx* ctx, uint32_t blas_id) {
    int rc = bvhgpu_blas_refit_async(ctx, blas_id, nullptr);
    if (rc) return rc;
    return finish(ctx);
}

int bvhgpu_blas_download_nodes(bvhgpu_ctx* ctx, uint32_t blas_id, bvhgpu_node* nodes) {
    if (!ctx || !nodes) return BVHGPU_ERR_INVALID_ARG;
    DeviceBlas* b = find_blas(ctx, blas_id);
    if (!b) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown BLAS %u", blas_id);
    std::vector<float> packed(8ull * b->nodes_used);
    CK(cudaStreamSynchronize(ctx->stream), "stream synchronize");
    CK(cudaMemcpy(packed.data(), b->nodes, 32ull * b->nodes_used, cudaMemcpyDeviceToHost), "download nodes");
    for (uint32_t i = 0; i < b->nodes_used; ++i) {
        const float* o = &packed[8ull * i];
        nodes[i].bounds_min[0] = o[0];
        nodes[i].bounds_min[1] = o[1];
        nodes[i].bounds_min[2] = o[2];
        std::memcpy(&nodes[i].left_first, &o[3], 4);
        nodes[i].bounds_max[0] = o[4];
        nodes[i].bounds_max[1] = o[5];
        nodes[i].bounds_max[2] = o[6];
        std::memcpy(&nodes[i].primitive_count, &o[7], 4);
    }
    return BVHGPU_OK;
}

int bvhgpu_blas_intersect_async(bvhgpu_ctx* ctx, uint32_t blas_id, const bvhgpu_ray* d_rays, uint32_t n,
                                bvhgpu_hit* d_hits, bvhgpu_stream s) {
    if (!ctx || (n && (!d_rays || !d_hits))) return BVHGPU_ERR_INVALID_ARG;
    if (n && (!rays_aligned(d_rays) || !hits_aligned(d_hits))) return misaligned(ctx, "blas_intersect_async");
    DeviceBlas* b = find_blas(ctx, blas_id);
    if (!b) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown BLAS %u", blas_id);
    CK(launch_trace_blas(ctx, *b, reinterpret_cast<const float4*>(d_rays), n, d_hits, pick(ctx, s)), "trace");
    return BVHGPU_OK;
}

int bvhgpu_blas_intersect(bvhgpu_ctx* ctx, uint32_t blas_id, const bvhgpu_ray* rays, uint32_t n, bvhgpu_hit* hits) {
    if (!ctx || (n && (!rays || !hits))) return BVHGPU_ERR_INVALID_ARG;
    DeviceBlas* b = find_blas(ctx, blas_id);
    if (!b) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown BLAS %u", blas_id);
    if (n == 0) return BVHGPU_OK;
    int rc = ensure(ctx, &ctx->stage_in, &ctx->stage_in_bytes, 32ull * n);
    if (!rc) rc = ensure(ctx, &ctx->stage_out, &ctx->stage_out_bytes, 20ull * n);
    if (rc) return rc;
    CK(cudaMemcpyAsync(ctx->stage_in, rays, 32ull * n, cudaMemcpyHostToDevice, ctx->stream), "upload rays");
    CK(launch_trace_blas(ctx, *b, static_cast<const float4*>(ctx->stage_in), n, ctx->stage_out, ctx->stream), "trace");
    CK(cudaMemcpyAsync(hits, ctx->stage_out, 20ull * n, cudaMemcpyDeviceToHost, ctx->stream), "download hits");
    return finish(ctx);
}

int bvhgpu_build_bvh_device(bvhgpu_ctx* ctx, bvhgpu_triangle* mesh, uint32_t n, bvhgpu_node* nodes_out,
                            uint32_t* nodes_used, uint32_t* perm_out) {
    if (!ctx || !mesh || !nodes_out || !nodes_used || n == 0 || n > 0x55555554u) return BVHGPU_ERR_INVALID_ARG;
    if (ctx->capturing) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "build_bvh_device: not allowed during capture");
    const char* what = "";
    int rc = build_bvh_device(ctx, reinterpret_cast<float*>(mesh), n, nodes_out, nodes_used, perm_out, &what);
    if (rc) return fail(ctx, rc, "GPU SAH build: %s", what);
    return BVHGPU_OK;
}

int bvhgpu_blas_build(bvhgpu_ctx* ctx, bvhgpu_triangle* mesh, uint32_t n, uint32_t* blas_id) {
    if (!ctx || !mesh || !blas_id || n == 0) return BVHGPU_ERR_INVALID_ARG;
    std::vector<bvhgpu_node> nodes(2ull * n);
    uint32_t used = 0;
    int rc = bvhgpu_build_bvh_device(ctx, mesh, n, nodes.data(), &used, nullptr);
    if (rc) return rc;
    return bvhgpu_blas_upload(ctx, nodes.data(), used, mesh, n, blas_id);
}

int bvhgpu_triangles_intersect_async(bvhgpu_ctx* ctx, const bvhgpu_triangle* d_tris, uint32_t ntris,
                                     const bvhgpu_ray* d_rays, uint32_t n, int mode, bvhgpu_hit* d_hits,
                                     bvhgpu_stream s) {
    if (!ctx || (n && (!d_rays || !d_hits)) || (ntris && !d_tris)) return BVHGPU_ERR_INVALID_ARG;
    if (n && (!rays_aligned(d_rays) || !hits_aligned(d_hits))) return misaligned(ctx, "triangles_intersect_async");
    if (mode != BVHGPU_LIST_CLOSEST && mode != BVHGPU_LIST_MUT)
        return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown triangle-list mode %d", mode);
    CK(launch_triangle_list(ctx, reinterpret_cast<const float*>(d_tris), ntris,
                            reinterpret_cast<const float4*>(d_rays), n, mode, d_hits, pick(ctx, s)),
       "triangle list");
    return BVHGPU_OK;
}

int bvhgpu_triangles_intersect(bvhgpu_ctx* ctx, const bvhgpu_triangle* tris, uint32_t ntris, const bvhgpu_ray* rays,
                               uint32_t n, int mode, bvhgpu_hit* hits) {
    if (!ctx || (n && (!rays || !hits)) || (ntris && !tris)) return BVHGPU_ERR_INVALID_ARG;
    if (n == 0) return BVHGPU_OK;
    int rc = ensure(ctx, &ctx->stage_in, &ctx->stage_in_bytes, 32ull * n);
    if (!rc) rc = ensure(ctx, &ctx->stage_out, &ctx->stage_out_bytes, 20ull * n);
    if (!rc) rc = ensure(ctx, &ctx->stage_out2, &ctx->stage_out2_bytes, 36ull * ntris + 16);
    if (rc) return rc;
    CK(cudaMemcpyAsync(ctx->stage_in, rays, 32ull * n, cudaMemcpyHostToDevice, ctx->stream), "upload rays");
    if (ntris)
        CK(cudaMemcpyAsync(ctx->stage_out2, tris, 36ull * ntris, cudaMemcpyHostToDevice, ctx->stream),
           "upload triangles");
    rc = bvhgpu_triangles_intersect_async(ctx, static_cast<const bvhgpu_triangle*>(ctx->stage_out2), ntris,
                                          static_cast<const bvhgpu_ray*>(ctx->stage_in), n, mode,
                                          static_cast<bvhgpu_hit*>(ctx->stage_out), nullptr);
    if (rc) return rc;
    CK(cudaMemcpyAsync(hits, ctx->stage_out, 20ull * n, cudaMemcpyDeviceToHost, ctx->stream), "download hits");
    return finish(ctx);
}

static int ensure_bounce(bvhgpu_ctx* ctx, uint32_t n) {
    if (ctx->bounce_cap >= n) return BVHGPU_OK;
    cudaFree(ctx->bounce_rays);
    cudaFree(ctx->bounce_pix);
    ctx->bounce_rays = nullptr;
    ctx->bounce_pix = nullptr;
    ctx->bounce_cap = 0;
    if (cudaMalloc(&ctx->bounce_rays, 32ull * n) != cudaSuccess ||
        cudaMalloc(&ctx->bounce_pix, 4ull * n) != cudaSuccess)
        return fail(ctx, BVHGPU_ERR_OUT_OF_MEMORY, "bounce queue of %u rays", n);
    ctx->bounce_cap = n;
    return BVHGPU_OK;
}

int bvhgpu_blas_trace_bounce_async(bvhgpu_ctx* ctx, uint32_t blas_id, const bvhgpu_ray* d_rays, uint32_t n,
                                   uint32_t seed, int mode, bvhgpu_hit* d_hits0, bvhgpu_hit* d_hits1,
                                   bvhgpu_stream s) {
    if (!ctx || (n && (!d_rays || !d_hits0 || !d_hits1))) return BVHGPU_ERR_INVALID_ARG;
    if (n && (!rays_aligned(d_rays) || !hits_aligned(d_hits0) || !hits_aligned(d_hits1)))
        return misaligned(ctx, "blas_trace_bounce_async");
    DeviceBlas* b = find_blas(ctx, blas_id);
    if (!b) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown BLAS %u", blas_id);
    const float4* r = reinterpret_cast<const float4*>(d_rays);
    if (mode == BVHGPU_MODE_PLAIN) {
        int rc = ensure_bounce(ctx, n);
        if (rc) return rc;
        CK(launch_bounce_plain(ctx, *b, r, n, seed, d_hits0, d_hits1, pick(ctx, s)), "bounce (plain)");
    } else if (mode == BVHGPU_MODE_PERSISTENT) {
        CK(launch_bounce_persistent(ctx, *b, r, n, seed, d_hits0, d_hits1, pick(ctx, s)), "bounce (persistent)");
    } else {
        return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown mode %d", mode);
    }
    return BVHGPU_OK;
}

// The device address of host memory the GPU can read and write in place (page-locked memory from
// cudaHostAlloc / bvhgpu_host_alloc), or null.
static void* mapped_device_ptr(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();  // clear: an unregistered pointer is not an error here
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// Writes one byte in every page of [p, p + bytes) from the CPU.  A GPU write to a page of ordinary
// host memory that the CPU never touched faults the page in through the CPU's page tables far more
// slowly than the CPU does (measured on the 1080p frame's fresh hit arrays: 28 ms against 1.2 ms).
// Only for buffers the launch then overwrites completely.
static void touch_pages(void* p, size_t bytes) {
    static const size_t page = static_cast<size_t>(sysconf(_SC_PAGESIZE));
    volatile char* c = static_cast<volatile char*>(p);
    const uintptr_t base = reinterpret_cast<uintptr_t>(p);
    for (size_t off = 0; off < bytes; off = ((base + off) / page + 1) * page - base) c[off] = 0;
}

// With page-locked host buffers the launch reads the rays and writes the hit records in place
// (over NVLink-C2C on Grace machines), so no copy phase precedes or follows it; on a device that
// reads and writes ordinary host memory coherently (cudaDevAttrPageableMemoryAccess) so does any
// host buffer, its hit pages touched first (1.15 ms against 1.93 ms staged for the 1080p frame).
// Otherwise: one upload, one launch, one download -- on GB300 the staged copies run at ~200 GB/s, while splitting
// the launch to overlap them costs more (each extra launch adds a ramp-up and a tail of
// ~0.3-0.5 ms).  The bounce count is reduced on the device either way.
int bvhgpu_blas_trace_bounce(bvhgpu_ctx* ctx, uint32_t blas_id, const bvhgpu_ray* rays, uint32_t n, uint32_t seed,
                             int mode, bvhgpu_hit* hits0, bvhgpu_hit* hits1, uint32_t* n_bounce) {
    if (!ctx || (n && (!rays || !hits0 || !hits1))) return BVHGPU_ERR_INVALID_ARG;
    if (n == 0) {
        if (n_bounce) *n_bounce = 0;
        return BVHGPU_OK;
    }
    uint32_t* d_count = ctx->d_scratch + 16;
    uint32_t* h_count = static_cast<uint32_t*>(ctx->host_word);
    DeviceBlas* b = find_blas(ctx, blas_id);
    if (!b) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown BLAS %u", blas_id);
    void* m_rays = mapped_device_ptr(rays);
    void* m_h0 = m_rays ? mapped_device_ptr(hits0) : nullptr;
    void* m_h1 = m_h0 ? mapped_device_ptr(hits1) : nullptr;
    if (!(rays_aligned(m_rays) && hits_aligned(m_h0) && hits_aligned(m_h1))) m_rays = m_h0 = m_h1 = nullptr;
    if (!(m_rays && m_h0 && m_h1) && ctx->pageable_access && rays_aligned(rays) && hits_aligned(hits0) &&
        hits_aligned(hits1)) {
        touch_pages(hits0, 20ull * n);
        touch_pages(hits1, 20ull * n);
        m_rays = const_cast<bvhgpu_ray*>(rays);
        m_h0 = hits0;
        m_h1 = hits1;
    }
    if (m_rays && m_h0 && m_h1 && mode == BVHGPU_MODE_PERSISTENT) {
        // the persistent launch counts its primary hits itself
        CK(cudaMemsetAsync(d_count, 0, sizeof(uint32_t), ctx->stream), "count");
        CK(launch_bounce_persistent(ctx, *b, static_cast<const float4*>(m_rays), n, seed, m_h0, m_h1, ctx->stream, 0,
                                    d_count),
           "bounce (persistent)");
        CK(cudaMemcpyAsync(h_count, d_count, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream), "count");
        const int rc = finish(ctx);
        if (rc) return rc;
        if (n_bounce) *n_bounce = *h_count;
        return BVHGPU_OK;
    }
    if (m_rays && m_h0 && m_h1) {
        int rc = bvhgpu_blas_trace_bounce_async(ctx, blas_id, static_cast<const bvhgpu_ray*>(m_rays), n, seed, mode,
                                                static_cast<bvhgpu_hit*>(m_h0), static_cast<bvhgpu_hit*>(m_h1),
                                                nullptr);
        if (rc) return rc;
        CK(cudaMemsetAsync(d_count, 0, sizeof(uint32_t), ctx->stream), "count");
        CK(launch_count_hits(ctx, m_h0, n, d_count, ctx->stream), "count");
        CK(cudaMemcpyAsync(h_count, d_count, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream), "count");
        rc = finish(ctx);
        if (rc) return rc;
        if (n_bounce) *n_bounce = *h_count;
        return BVHGPU_OK;
    }
    int rc = ensure(ctx, &ctx->stage_in, &ctx->stage_in_bytes, 32ull * n);
    if (!rc) rc = ensure(ctx, &ctx->stage_out, &ctx->stage_out_bytes, 20ull * n);
    if (!rc) rc = ensure(ctx, &ctx->stage_out2, &ctx->stage_out2_bytes, 20ull * n);
    if (rc) return rc;
    CK(cudaMemcpyAsync(ctx->stage_in, rays, 32ull * n, cudaMemcpyHostToDevice, ctx->stream), "upload rays");
    rc = bvhgpu_blas_trace_bounce_async(ctx, blas_id, static_cast<const bvhgpu_ray*>(ctx->stage_in), n, seed, mode,
                                        static_cast<bvhgpu_hit*>(ctx->stage_out),
                                        static_cast<bvhgpu_hit*>(ctx->stage_out2), nullptr);
    if (rc) return rc;
    CK(cudaMemsetAsync(d_count, 0, sizeof(uint32_t), ctx->stream), "count");
    CK(launch_count_hits(ctx, ctx->stage_out, n, d_count, ctx->stream), "count");
    CK(cudaMemcpyAsync(hits0, ctx->stage_out, 20ull * n, cudaMemcpyDeviceToHost, ctx->stream), "download hits");
    CK(cudaMemcpyAsync(hits1, ctx->stage_out2, 20ull * n, cudaMemcpyDeviceToHost, ctx->stream), "download hits");
    CK(cudaMemcpyAsync(h_count, d_count, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream), "count");
    rc = finish(ctx);
    if (rc) return rc;
    if (n_bounce) *n_bounce = *h_count;
    return BVHGPU_OK;
}

int bvhgpu_blas_bounce_rays(bvhgpu_ctx* ctx, uint32_t blas_id, const bvhgpu_ray* rays, uint32_t n, uint32_t seed,
                            bvhgpu_ray* out, uint8_t* valid) {
    if (!ctx || (n && (!rays || !out || !valid))) return BVHGPU_ERR_INVALID_ARG;
    DeviceBlas* b = find_blas(ctx, blas_id);
    if (!b) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown BLAS %u", blas_id);
    if (n == 0) return BVHGPU_OK;
    void *d_rays = nullptr, *d_hits = nullptr, *d_out = nullptr, *d_valid = nullptr;
    auto done = [&]() {
        cudaFree(d_rays);
        cudaFree(d_hits);
        cudaFree(d_out);
        cudaFree(d_valid);
    };
    if (cudaMalloc(&d_rays, 32ull * n) != cudaSuccess || cudaMalloc(&d_hits, 20ull * n) != cudaSuccess ||
        cudaMalloc(&d_out, 32ull * n) != cudaSuccess || cudaMalloc(&d_valid, n) != cudaSuccess) {
        done();
        return fail(ctx, BVHGPU_ERR_OUT_OF_MEMORY, "bounce_rays buffers");
    }
    cudaError_t e;
    if ((e = cudaMemcpyAsync(d_rays, rays, 32ull * n, cudaMemcpyHostToDevice, ctx->stream)) != cudaSuccess ||
        (e = launch_trace_blas(ctx, *b, static_cast<const float4*>(d_rays), n, d_hits, ctx->stream)) != cudaSuccess ||
        (e = launch_bounce_rays(ctx, *b, static_cast<const float4*>(d_rays), d_hits, n, seed,
                                static_cast<float4*>(d_out), static_cast<uint8_t*>(d_valid), ctx->stream)) !=
            cudaSuccess ||
        (e = cudaMemcpyAsync(out, d_out, 32ull * n, cudaMemcpyDeviceToHost, ctx->stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(valid, d_valid, n, cudaMemcpyDeviceToHost, ctx->stream)) != cudaSuccess) {
        done();
        return cuda_fail(ctx, e, "bounce_rays");
    }
    int rc = finish(ctx);
    done();
    return rc;
}

int bvhgpu_trace_batch_async(bvhgpu_ctx* ctx, const bvhgpu_batch_item* items, uint32_t nitems,
                             const bvhgpu_ray* d_rays, uint32_t nrays, int mode, bvhgpu_hit* d_hits, bvhgpu_stream s) {
    if (!ctx || (nitems && (!items || !d_rays || !d_hits))) return BVHGPU_ERR_INVALID_ARG;
    if (nitems && (!rays_aligned(d_rays) || !hits_aligned(d_hits))) return misaligned(ctx, "trace_batch_async");
    if (mode != BVHGPU_MODE_PLAIN && mode != BVHGPU_MODE_PERSISTENT)
        return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown mode %d", mode);
    std::vector<const DeviceBlas*> blases(nitems);
    for (uint32_t i = 0; i < nitems; ++i) {
        blases[i] = find_blas(ctx, items[i].blas);
        if (!blases[i]) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "batch item %u: unknown BLAS %u", i, items[i].blas);
        if ((uint64_t)items[i].ray_offset + items[i].ray_count > nrays)
            return fail(ctx, BVHGPU_ERR_INVALID_ARG, "batch item %u: rays past %u", i, nrays);
    }
    // a new item list is uploaded synchronously (stream synchronize, allocation, copy), which a stream
    // capture cannot record: trace a new list once before capturing it
    if (mode == BVHGPU_MODE_PERSISTENT && nitems && ctx->capturing && !batch_table_current(ctx, items, nitems))
        return fail(ctx, BVHGPU_ERR_INVALID_ARG,
                    "trace_batch: a new item list cannot be set up during graph capture (trace it once first)");
    CK(launch_trace_batch(ctx, blases, items, nitems, reinterpret_cast<const float4*>(d_rays), nrays, mode, d_hits,
                          pick(ctx, s)),
       "trace batch");
    return BVHGPU_OK;
}

int bvhgpu_trace_batch(bvhgpu_ctx* ctx, const bvhgpu_batch_item* items, uint32_t nitems, const bvhgpu_ray* rays,
                       uint32_t nrays, int mode, bvhgpu_hit* hits) {
    if (!ctx || (nrays && (!rays || !hits))) return BVHGPU_ERR_INVALID_ARG;
    if (nrays == 0) return BVHGPU_OK;
    int rc = ensure(ctx, &ctx->stage_in, &ctx->stage_in_bytes, 32ull * nrays);
    if (!rc) rc = ensure(ctx, &ctx->stage_out, &ctx->stage_out_bytes, 20ull * nrays);
    if (rc) return rc;
    CK(cudaMemcpyAsync(ctx->stage_in, rays, 32ull * nrays, cudaMemcpyHostToDevice, ctx->stream), "upload rays");
    rc = bvhgpu_trace_batch_async(ctx, items, nitems, static_cast<const bvhgpu_ray*>(ctx->stage_in), nrays, mode,
                                  static_cast<bvhgpu_hit*>(ctx->stage_out), nullptr);
    if (rc) return rc;
    CK(cudaMemcpyAsync(hits, ctx->stage_out, 20ull * nrays, cudaMemcpyDeviceToHost, ctx->stream), "download hits");
    return finish(ctx);
}

// ---- scenes --------------------------------------------------------------------------------------

int bvhgpu_scene_create(bvhgpu_ctx* ctx, const uint32_t* blas_ids, uint32_t nobjects, uint32_t* scene_id) {
    if (!ctx || !blas_ids || !scene_id || nobjects == 0)
        return fail(ctx, BVHGPU_ERR_INVALID_ARG, "scene_create: empty scene");
    if (nobjects > kMaxSceneObjects)
        return fail(ctx, BVHGPU_ERR_INVALID_ARG, "scene_create: at most %u objects (16-bit TLAS node indices)",
                    kMaxSceneObjects);
    DeviceScene sc;
    sc.nobjects = nobjects;
    sc.blas_ids.assign(blas_ids, blas_ids + nobjects);
    std::vector<uint32_t> obj_blas(nobjects);
    std::vector<GBlas> table;
    for (uint32_t i = 0; i < nobjects; ++i) {
        DeviceBlas* b = find_blas(ctx, blas_ids[i]);
        if (!b) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "scene_create: unknown BLAS %u", blas_ids[i]);
        auto it = std::find(sc.table_blas.begin(), sc.table_blas.end(), blas_ids[i]);
        if (it == sc.table_blas.end()) {
            sc.table_blas.push_back(blas_ids[i]);
            GBlas g;
            g.nodes = b->nodes;
            g.tris = b->tris;
            g.pairs = b->pairs;
            g.hx = b->hx;
            g.cones = b->cones;
            g.nodes_used = b->nodes_used;
            g.ntris = b->ntris;
            g.root_count = b->root_count;
            g.root_first = b->root_first;
            table.push_back(g);
            obj_blas[i] = (uint32_t)table.size() - 1;
        } else {
            obj_blas[i] = (uint32_t)(it - sc.table_blas.begin());
        }
    }
    sc.nblas = (uint32_t)table.size();
    std::vector<float> ident(16ull * nobjects, 0.0f);
    for (uint32_t i = 0; i < nobjects; ++i)
        for (int k = 0; k < 4; ++k) ident[16ull * i + 5 * k] = 1.0f;
    cudaError_t e;
    if ((e = cudaMalloc(&sc.xf, 64ull * nobjects)) != cudaSuccess ||
        (e = cudaMalloc(&sc.inv, 64ull * nobjects)) != cudaSuccess ||
        (e = cudaMalloc(&sc.obj_blas, 4ull * nobjects)) != cudaSuccess ||
        (e = cudaMalloc(&sc.blas_table, sizeof(GBlas) * table.size())) != cudaSuccess ||
        (e = cudaMalloc(&sc.tlas, 64ull * nobjects)) != cudaSuccess ||
        (nobjects > kTlasSharedObjects && (e = cudaMalloc(&sc.tlas_work, tlas_smem_bytes(nobjects))) != cudaSuccess)) {
        free_scene(sc);
        return fail(ctx, BVHGPU_ERR_OUT_OF_MEMORY, "scene_create: %s", cudaGetErrorString(e));
    }
    if ((e = cudaMemcpy(sc.xf, ident.data(), 64ull * nobjects, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(sc.inv, ident.data(), 64ull * nobjects, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(sc.obj_blas, obj_blas.data(), 4ull * nobjects, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(sc.blas_table, table.data(), sizeof(GBlas) * table.size(), cudaMemcpyHostToDevice)) !=
            cudaSuccess) {
        free_scene(sc);
        return cuda_fail(ctx, e, "scene_create");
    }
    uint32_t id = ctx->next_scene++;
    ctx->scenes[id] = sc;
    *scene_id = id;
    return bvhgpu_scene_rebuild(ctx, id);
}

int bvhgpu_scene_free(bvhgpu_ctx* ctx, uint32_t scene_id) {
    if (!ctx) return BVHGPU_ERR_INVALID_ARG;
    DeviceScene* sc = find_scene(ctx, scene_id);
    if (!sc) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown scene %u", scene_id);
    cudaStreamSynchronize(ctx->stream);
    free_scene(*sc);
    ctx->scenes.erase(scene_id);
    return BVHGPU_OK;
}

int bvhgpu_scene_set_transforms_async(bvhgpu_ctx* ctx, uint32_t scene_id, const float* d_xf, const float* d_inv,
                                      bvhgpu_stream s) {
    if (!ctx || !d_xf || !d_inv) return BVHGPU_ERR_INVALID_ARG;
    DeviceScene* sc = find_scene(ctx, scene_id);
    if (!sc) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown scene %u", scene_id);
    CK(cudaMemcpyAsync(sc->xf, d_xf, 64ull * sc->nobjects, cudaMemcpyDeviceToDevice, pick(ctx, s)), "transforms");
    CK(cudaMemcpyAsync(sc->inv, d_inv, 64ull * sc->nobjects, cudaMemcpyDeviceToDevice, pick(ctx, s)), "inverses");
    return BVHGPU_OK;
}

int bvhgpu_scene_set_transforms(bvhgpu_ctx* ctx, uint32_t scene_id, const float* xf, const float* inv) {
    if (!ctx || !xf || !inv) return BVHGPU_ERR_INVALID_ARG;
    DeviceScene* sc = find_scene(ctx, scene_id);
    if (!sc) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown scene %u", scene_id);
    CK(cudaStreamSynchronize(ctx->stream), "stream synchronize");
    CK(cudaMemcpy(sc->xf, xf, 64ull * sc->nobjects, cudaMemcpyHostToDevice), "transforms");
    CK(cudaMemcpy(sc->inv, inv, 64ull * sc->nobjects, cudaMemcpyHostToDevice), "inverses");
    return BVHGPU_OK;
}

int bvhgpu_scene_rebuild_async(bvhgpu_ctx* ctx, uint32_t scene_id, bvhgpu_stream s) {
    if (!ctx) return BVHGPU_ERR_INVALID_ARG;
    DeviceScene* sc = find_scene(ctx, scene_id);
    if (!sc) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown scene %u", scene_id);
    CK(launch_tlas_rebuild(ctx, *sc, pick(ctx, s)), "TLAS rebuild");
    sc->tlas_nodes_used = 2 * sc->nobjects;
    return BVHGPU_OK;
}

int bvhgpu_scene_rebuild(bvhgpu_ctx* ctx, uint32_t scene_id) {
    int rc = bvhgpu_scene_rebuild_async(ctx, scene_id, nullptr);
    if (rc) return rc;
    rc = finish(ctx);
    if (rc) return rc;
    uint32_t status[2] = {0, 0};
    CK(cudaMemcpy(status, ctx->d_scratch + 8, sizeof(status), cudaMemcpyDeviceToHost), "TLAS status");
    if (status[1]) return fail(ctx, BVHGPU_ERR_BUILD, "TLAS rebuild: the reference would panic (NaN bounds)");
    find_scene(ctx, scene_id)->tlas_nodes_used = status[0];
    return BVHGPU_OK;
}

int bvhgpu_scene_download_tlas(bvhgpu_ctx* ctx, uint32_t scene_id, bvhgpu_tlas_node* nodes, uint32_t* nodes_used) {
    if (!ctx || !nodes) return BVHGPU_ERR_INVALID_ARG;
    DeviceScene* sc = find_scene(ctx, scene_id);
    if (!sc) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown scene %u", scene_id);
    std::vector<float> packed(16ull * sc->nobjects);
    CK(cudaStreamSynchronize(ctx->stream), "stream synchronize");
    CK(cudaMemcpy(packed.data(), sc->tlas, 64ull * sc->nobjects, cudaMemcpyDeviceToHost), "download TLAS");
    for (uint32_t i = 0; i < 2 * sc->nobjects; ++i) {
        const float* o = &packed[8ull * i];
        for (int k = 0; k < 3; ++k) {
            nodes[i].bounds_min[k] = o[k];
            nodes[i].bounds_max[k] = o[4 + k];
        }
        std::memcpy(&nodes[i].left_right, &o[3], 4);
        std::memcpy(&nodes[i].blas, &o[7], 4);
    }
    if (nodes_used) *nodes_used = sc->tlas_nodes_used;
    return BVHGPU_OK;
}

int bvhgpu_scene_intersect_async(bvhgpu_ctx* ctx, uint32_t scene_id, const bvhgpu_ray* d_rays, uint32_t n,
                                 bvhgpu_hit* d_hits, bvhgpu_stream s) {
    if (!ctx || (n && (!d_rays || !d_hits))) return BVHGPU_ERR_INVALID_ARG;
    if (n && (!rays_aligned(d_rays) || !hits_aligned(d_hits))) return misaligned(ctx, "scene_intersect_async");
    DeviceScene* sc = find_scene(ctx, scene_id);
    if (!sc) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown scene %u", scene_id);
    CK(launch_trace_scene(ctx, *sc, reinterpret_cast<const float4*>(d_rays), n, d_hits, pick(ctx, s)), "trace scene");
    return BVHGPU_OK;
}

int bvhgpu_scene_intersect(bvhgpu_ctx* ctx, uint32_t scene_id, const bvhgpu_ray* rays, uint32_t n, bvhgpu_hit* hits) {
    if (!ctx || (n && (!rays || !hits))) return BVHGPU_ERR_INVALID_ARG;
    if (n == 0) return BVHGPU_OK;
    int rc = ensure(ctx, &ctx->stage_in, &ctx->stage_in_bytes, 32ull * n);
    if (!rc) rc = ensure(ctx, &ctx->stage_out, &ctx->stage_out_bytes, 20ull * n);
    if (rc) return rc;
    CK(cudaMemcpyAsync(ctx->stage_in, rays, 32ull * n, cudaMemcpyHostToDevice, ctx->stream), "upload rays");
    rc = bvhgpu_scene_intersect_async(ctx, scene_id, static_cast<const bvhgpu_ray*>(ctx->stage_in), n,
                                      static_cast<bvhgpu_hit*>(ctx->stage_out), nullptr);
    if (rc) return rc;
    CK(cudaMemcpyAsync(hits, ctx->stage_out, 20ull * n, cudaMemcpyDeviceToHost, ctx->stream), "download hits");
    return finish(ctx);
}

// ---- differentiable Lambertian render ---------------------------------------------------------------

int bvhgpu_mesh_create(bvhgpu_ctx* ctx, uint32_t blas_id, const uint32_t* faces, uint32_t nfaces, const float* verts,
                       const float* vnormals, uint32_t nverts, uint32_t* mesh_id) {
    if (!ctx || !faces || !verts || !vnormals || !mesh_id || nverts == 0) return BVHGPU_ERR_INVALID_ARG;
    DeviceBlas* b = find_blas(ctx, blas_id);
    if (!b) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown BLAS %u", blas_id);
    if (nfaces != b->ntris) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "mesh has %u faces, BLAS %u triangles", nfaces, b->ntris);
    for (uint64_t i = 0; i < 3ull * nfaces; ++i)
        if (faces[i] >= nverts) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "face index %u past %u vertices", faces[i], nverts);
    DeviceMesh m;
    m.blas = blas_id;
    m.nfaces = nfaces;
    m.nverts = nverts;
    cudaError_t e;
    if ((e = cudaMalloc(&m.faces, 12ull * nfaces)) != cudaSuccess || (e = cudaMalloc(&m.verts, 12ull * nverts)) != cudaSuccess ||
        (e = cudaMalloc(&m.vnormals, 12ull * nverts)) != cudaSuccess) {
        free_mesh(m);
        return fail(ctx, BVHGPU_ERR_OUT_OF_MEMORY, "mesh_create: %s", cudaGetErrorString(e));
    }
    if ((e = cudaMemcpy(m.faces, faces, 12ull * nfaces, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(m.verts, verts, 12ull * nverts, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(m.vnormals, vnormals, 12ull * nverts, cudaMemcpyHostToDevice)) != cudaSuccess) {
        free_mesh(m);
        return cuda_fail(ctx, e, "mesh_create");
    }
    uint32_t id = ctx->next_mesh++;
    ctx->meshes[id] = m;
    *mesh_id = id;
    return BVHGPU_OK;
}

int bvhgpu_mesh_free(bvhgpu_ctx* ctx, uint32_t mesh_id) {
    if (!ctx) return BVHGPU_ERR_INVALID_ARG;
    DeviceMesh* m = find_mesh(ctx, mesh_id);
    if (!m) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown mesh %u", mesh_id);
    cudaStreamSynchronize(ctx->stream);
    free_mesh(*m);
    ctx->meshes.erase(mesh_id);
    return BVHGPU_OK;
}

int bvhgpu_mesh_vertices(bvhgpu_ctx* ctx, uint32_t mesh_id, float** d_verts) {
    if (!ctx || !d_verts) return BVHGPU_ERR_INVALID_ARG;
    DeviceMesh* m = find_mesh(ctx, mesh_id);
    if (!m) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown mesh %u", mesh_id);
    *d_verts = m->verts;
    return BVHGPU_OK;
}

int bvhgpu_mesh_update_async(bvhgpu_ctx* ctx, uint32_t mesh_id, bvhgpu_stream s) {
    if (!ctx) return BVHGPU_ERR_INVALID_ARG;
    DeviceMesh* m = find_mesh(ctx, mesh_id);
    if (!m) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown mesh %u", mesh_id);
    DeviceBlas* b = find_blas(ctx, m->blas);
    if (!b) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "mesh %u: BLAS %u was freed", mesh_id, m->blas);
    CK(launch_mesh_update(ctx, *m, *b, pick(ctx, s)), "mesh update");
    return BVHGPU_OK;
}

int bvhgpu_mesh_set_vertices(bvhgpu_ctx* ctx, uint32_t mesh_id, const float* verts) {
    if (!ctx || !verts) return BVHGPU_ERR_INVALID_ARG;
    DeviceMesh* m = find_mesh(ctx, mesh_id);
    if (!m) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown mesh %u", mesh_id);
    CK(cudaStreamSynchronize(ctx->stream), "stream synchronize");
    CK(cudaMemcpy(m->verts, verts, 12ull * m->nverts, cudaMemcpyHostToDevice), "upload vertices");
    int rc = bvhgpu_mesh_update_async(ctx, mesh_id, nullptr);
    if (rc) return rc;
    return finish(ctx);
}

int bvhgpu_lambert_forward_async(bvhgpu_ctx* ctx, uint32_t mesh_id, const bvhgpu_ray* d_rays, uint32_t n,
                                 const float light[3], float* d_image, bvhgpu_hit* d_hits, bvhgpu_stream s) {
    if (!ctx || !light || (n && (!d_rays || !d_image || !d_hits))) return BVHGPU_ERR_INVALID_ARG;
    if (n && (!rays_aligned(d_rays) || !hits_aligned(d_hits) || !hits_aligned(d_image)))
        return misaligned(ctx, "lambert_forward_async");
    DeviceMesh* m = find_mesh(ctx, mesh_id);
    if (!m) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown mesh %u", mesh_id);
    DeviceBlas* b = find_blas(ctx, m->blas);
    if (!b) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "mesh %u: BLAS %u was freed", mesh_id, m->blas);
    CK(launch_lambert_forward(ctx, *m, *b, reinterpret_cast<const float4*>(d_rays), n, light, d_image, d_hits,
                              pick(ctx, s)),
       "lambert forward");
    return BVHGPU_OK;
}

int bvhgpu_mse_loss(bvhgpu_ctx* ctx, const float* d_image, const float* d_target, uint32_t n, double* loss) {
    if (!ctx || !loss || (n && (!d_image || !d_target))) return BVHGPU_ERR_INVALID_ARG;
    if (n == 0) {
        *loss = 0.0;
        return BVHGPU_OK;
    }
    size_t nb = (n + 255) / 256;
    if (ctx->mse_partials_cap < nb) {
        cudaFree(ctx->mse_partials);
        ctx->mse_partials = nullptr;
        ctx->mse_partials_cap = 0;
        CK(cudaMalloc(&ctx->mse_partials, 8 * nb), "loss partials");
        ctx->mse_partials_cap = nb;
    }
    CK(launch_mse_partials(ctx, d_image, d_target, n, ctx->mse_partials, ctx->stream), "loss");
    std::vector<double> parts(nb);
    CK(cudaMemcpyAsync(parts.data(), ctx->mse_partials, 8 * nb, cudaMemcpyDeviceToHost, ctx->stream), "loss copy");
    int rc = finish(ctx);
    if (rc) return rc;
    double sum = 0.0;
    for (double p : parts) sum += p;
    *loss = sum / (double)n;
    return BVHGPU_OK;
}

int bvhgpu_lambert_adjoint_async(bvhgpu_ctx* ctx, uint32_t mesh_id, const bvhgpu_ray* d_rays, uint32_t n,
                                 const float light[3], const bvhgpu_hit* d_hits, const float* d_image,
                                 const float* d_target, float* d_grad, bvhgpu_stream s) {
    if (!ctx || !light || (n && (!d_rays || !d_hits || !d_image || !d_target || !d_grad))) return BVHGPU_ERR_INVALID_ARG;
    if (n && (!rays_aligned(d_rays) || !hits_aligned(d_hits))) return misaligned(ctx, "lambert_adjoint_async");
    DeviceMesh* m = find_mesh(ctx, mesh_id);
    if (!m) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown mesh %u", mesh_id);
    CK(launch_lambert_adjoint(ctx, *m, reinterpret_cast<const float4*>(d_rays), n, light, d_hits, d_image, d_target,
                              d_grad, pick(ctx, s)),
       "lambert adjoint");
    return BVHGPU_OK;
}

int bvhgpu_mesh_sgd_step_async(bvhgpu_ctx* ctx, uint32_t mesh_id, float* d_grad, float lr, bvhgpu_stream s) {
    if (!ctx || !d_grad) return BVHGPU_ERR_INVALID_ARG;
    DeviceMesh* m = find_mesh(ctx, mesh_id);
    if (!m) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown mesh %u", mesh_id);
    CK(launch_sgd(ctx, *m, d_grad, lr, pick(ctx, s)), "sgd step");
    return BVHGPU_OK;
}

// ---- instanced frames ----------------------------------------------------------------------------

int bvhgpu_scene_trace_bounce_async(bvhgpu_ctx* ctx, uint32_t scene_id, const bvhgpu_ray* d_rays, uint32_t n,
                                    uint32_t seed, bvhgpu_hit* d_hits0, bvhgpu_hit* d_hits1, bvhgpu_stream s) {
    if (!ctx || (n && (!d_rays || !d_hits0 || !d_hits1))) return BVHGPU_ERR_INVALID_ARG;
    if (n && (!rays_aligned(d_rays) || !hits_aligned(d_hits0) || !hits_aligned(d_hits1)))
        return misaligned(ctx, "scene_trace_bounce_async");
    DeviceScene* sc = find_scene(ctx, scene_id);
    if (!sc) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown scene %u", scene_id);
    CK(launch_scene_bounce(ctx, *sc, reinterpret_cast<const float4*>(d_rays), n, seed, d_hits0, d_hits1, pick(ctx, s)),
       "scene bounce");
    return BVHGPU_OK;
}

int bvhgpu_scene_bounce_rays(bvhgpu_ctx* ctx, uint32_t scene_id, const bvhgpu_ray* rays, uint32_t n, uint32_t seed,
                             bvhgpu_ray* out, uint8_t* valid) {
    if (!ctx || (n && (!rays || !out || !valid))) return BVHGPU_ERR_INVALID_ARG;
    DeviceScene* sc = find_scene(ctx, scene_id);
    if (!sc) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown scene %u", scene_id);
    if (n == 0) return BVHGPU_OK;
    void *d_rays = nullptr, *d_hits = nullptr, *d_out = nullptr, *d_valid = nullptr;
    auto done = [&]() {
        cudaFree(d_rays);
        cudaFree(d_hits);
        cudaFree(d_out);
        cudaFree(d_valid);
    };
    if (cudaMalloc(&d_rays, 32ull * n) != cudaSuccess || cudaMalloc(&d_hits, 20ull * n) != cudaSuccess ||
        cudaMalloc(&d_out, 32ull * n) != cudaSuccess || cudaMalloc(&d_valid, n) != cudaSuccess) {
        done();
        return fail(ctx, BVHGPU_ERR_OUT_OF_MEMORY, "scene_bounce_rays buffers");
    }
    cudaError_t e;
    if ((e = cudaMemcpyAsync(d_rays, rays, 32ull * n, cudaMemcpyHostToDevice, ctx->stream)) != cudaSuccess ||
        (e = launch_trace_scene(ctx, *sc, static_cast<const float4*>(d_rays), n, d_hits, ctx->stream)) != cudaSuccess ||
        (e = launch_scene_bounce_rays(ctx, *sc, static_cast<const float4*>(d_rays), d_hits, n, seed,
                                      static_cast<float4*>(d_out), static_cast<uint8_t*>(d_valid), ctx->stream)) !=
            cudaSuccess ||
        (e = cudaMemcpyAsync(out, d_out, 32ull * n, cudaMemcpyDeviceToHost, ctx->stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(valid, d_valid, n, cudaMemcpyDeviceToHost, ctx->stream)) != cudaSuccess) {
        done();
        return cuda_fail(ctx, e, "scene_bounce_rays");
    }
    int rc = finish(ctx);
    done();
    return rc;
}

int bvhgpu_scene_download_transforms(bvhgpu_ctx* ctx, uint32_t scene_id, float* xf, float* inv) {
    if (!ctx || !xf || !inv) return BVHGPU_ERR_INVALID_ARG;
    DeviceScene* sc = find_scene(ctx, scene_id);
    if (!sc) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown scene %u", scene_id);
    CK(cudaStreamSynchronize(ctx->stream), "stream synchronize");
    CK(cudaMemcpy(xf, sc->xf, 64ull * sc->nobjects, cudaMemcpyDeviceToHost), "download transforms");
    CK(cudaMemcpy(inv, sc->inv, 64ull * sc->nobjects, cudaMemcpyDeviceToHost), "download inverses");
    return BVHGPU_OK;
}

int bvhgpu_mesh_wobble_async(bvhgpu_ctx* ctx, uint32_t mesh_id, const float* d_dirs, const float* d_r0,
                             const float* d_phase, float amp, float freq, const float* d_time, bvhgpu_stream s) {
    if (!ctx || !d_dirs || !d_r0 || !d_phase || !d_time) return BVHGPU_ERR_INVALID_ARG;
    DeviceMesh* m = find_mesh(ctx, mesh_id);
    if (!m) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown mesh %u", mesh_id);
    CK(launch_wobble(ctx, m->verts, d_dirs, d_r0, d_phase, m->nverts, amp, freq, d_time, pick(ctx, s)), "wobble");
    return BVHGPU_OK;
}

int bvhgpu_scene_animate_async(bvhgpu_ctx* ctx, uint32_t scene_id, const float* d_rot0, const float* d_axis,
                               const float* d_omega, const float* d_scale, const float* d_trans, const float* d_time,
                               bvhgpu_stream s) {
    if (!ctx || !d_rot0 || !d_axis || !d_omega || !d_scale || !d_trans || !d_time) return BVHGPU_ERR_INVALID_ARG;
    DeviceScene* sc = find_scene(ctx, scene_id);
    if (!sc) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown scene %u", scene_id);
    CK(launch_animate_instances(ctx, *sc, d_rot0, d_axis, d_omega, d_scale, d_trans, d_time, pick(ctx, s)),
       "animate instances");
    return BVHGPU_OK;
}

int bvhgpu_advance_time_async(bvhgpu_ctx* ctx, float* d_time, float dt, bvhgpu_stream s) {
    if (!ctx || !d_time) return BVHGPU_ERR_INVALID_ARG;
    CK(launch_advance_time(ctx, d_time, dt, pick(ctx, s)), "advance time");
    return BVHGPU_OK;
}

int bvhgpu_graph_begin(bvhgpu_ctx* ctx) {
    if (!ctx || ctx->capturing) return BVHGPU_ERR_INVALID_ARG;
    CK(cudaStreamSynchronize(ctx->stream), "stream synchronize");
    ctx->profiling_before_capture = ctx->profiling;
    ctx->profiling = false;  // no timing events inside a captured graph
    CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
    ctx->capturing = true;
    return BVHGPU_OK;
}

int bvhgpu_graph_end(bvhgpu_ctx* ctx, uint32_t* graph_id) {
    if (!ctx || !graph_id || !ctx->capturing) return BVHGPU_ERR_INVALID_ARG;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    ctx->capturing = false;
    ctx->profiling = ctx->profiling_before_capture;
    if (e != cudaSuccess) return cuda_fail(ctx, e, "end capture");
    cudaGraphExec_t ex = nullptr;
    e = cudaGraphInstantiate(&ex, g, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        return cuda_fail(ctx, e, "instantiate graph");
    }
    uint32_t id = ctx->next_graph++;
    ctx->graphs[id] = {g, ex};
    *graph_id = id;
    return BVHGPU_OK;
}

int bvhgpu_graph_launch(bvhgpu_ctx* ctx, uint32_t graph_id) {
    if (!ctx) return BVHGPU_ERR_INVALID_ARG;
    auto it = ctx->graphs.find(graph_id);
    if (it == ctx->graphs.end()) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown graph %u", graph_id);
    CK(cudaGraphLaunch(it->second.second, ctx->stream), "graph launch");
    g_launches++;
    return BVHGPU_OK;
}

int bvhgpu_graph_free(bvhgpu_ctx* ctx, uint32_t graph_id) {
    if (!ctx) return BVHGPU_ERR_INVALID_ARG;
    auto it = ctx->graphs.find(graph_id);
    if (it == ctx->graphs.end()) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown graph %u", graph_id);
    cudaStreamSynchronize(ctx->stream);
    cudaGraphExecDestroy(it->second.second);
    cudaGraphDestroy(it->second.first);
    ctx->graphs.erase(it);
    return BVHGPU_OK;
}

// ---- render -------------------------------------------------------------------------------------

int bvhgpu_render(bvhgpu_ctx* ctx, uint32_t blas_id, const bvhgpu_camera* camera, int width, int height,
                  int accumulator, const float* acc_params, int shader, const float* shader_params,
                  const float* normals, uint8_t* rgba, uint64_t* rays_traced) {
    if (!ctx || !camera || !rgba || width <= 0 || height <= 0) return BVHGPU_ERR_INVALID_ARG;
    if (accumulator < 0 || accumulator > 3 || shader < 0 || shader > 2)
        return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown accumulator %d or shader %d", accumulator, shader);
    if ((accumulator == BVHGPU_ACC_INTERSECTION || accumulator == BVHGPU_ACC_NORMAL) && !acc_params)
        return fail(ctx, BVHGPU_ERR_INVALID_ARG, "accumulator needs parameters");
    if ((shader == BVHGPU_SHADER_INTERSECTION || shader == BVHGPU_SHADER_DEPTH) && !shader_params)
        return fail(ctx, BVHGPU_ERR_INVALID_ARG, "shader needs parameters");
    DeviceBlas* b = find_blas(ctx, blas_id);
    if (!b) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown BLAS %u", blas_id);
    if (accumulator == BVHGPU_ACC_NORMAL && !normals) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "normals required");
    size_t px = (size_t)width * height;
    int rc = ensure(ctx, &ctx->stage_out, &ctx->stage_out_bytes, 4 * px);
    if (!rc && normals) rc = ensure(ctx, &ctx->stage_in, &ctx->stage_in_bytes, 36ull * b->ntris);
    if (rc) return rc;
    if (normals)
        CK(cudaMemcpyAsync(ctx->stage_in, normals, 36ull * b->ntris, cudaMemcpyHostToDevice, ctx->stream), "normals");
    CK(launch_render(ctx, *b, *camera, width, height, accumulator, acc_params, shader, shader_params,
                     normals ? static_cast<const float*>(ctx->stage_in) : nullptr, nullptr, nullptr, 0, 0,
                     static_cast<uint8_t*>(ctx->stage_out), ctx->stream),
       "render");
    CK(cudaMemcpyAsync(rgba, ctx->stage_out, 4 * px, cudaMemcpyDeviceToHost, ctx->stream), "download frame");
    rc = finish(ctx);
    if (rc) return rc;
    if (rays_traced) *rays_traced = px;
    return BVHGPU_OK;
}

int bvhgpu_render_textured(bvhgpu_ctx* ctx, uint32_t blas_id, const bvhgpu_camera* camera, int width, int height,
                           const float* tex_coords, const uint8_t* texels, uint32_t tex_w, uint32_t tex_h,
                           int shader, const float* shader_params, uint8_t* rgba, uint64_t* rays_traced) {
    if (!ctx || !camera || !rgba || width <= 0 || height <= 0 || !tex_coords || !texels || tex_w == 0 ||
        tex_h == 0)
        return BVHGPU_ERR_INVALID_ARG;
    if (shader < 0 || shader > 2) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown shader %d", shader);
    if ((shader == BVHGPU_SHADER_INTERSECTION || shader == BVHGPU_SHADER_DEPTH) && !shader_params)
        return fail(ctx, BVHGPU_ERR_INVALID_ARG, "shader needs parameters");
    DeviceBlas* b = find_blas(ctx, blas_id);
    if (!b) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown BLAS %u", blas_id);
    const size_t px = (size_t)width * height, tc_bytes = 24ull * b->ntris, tex_bytes = 3ull * tex_w * tex_h;
    int rc = ensure(ctx, &ctx->stage_out, &ctx->stage_out_bytes, 4 * px);
    if (!rc) rc = ensure(ctx, &ctx->stage_in, &ctx->stage_in_bytes, tc_bytes + tex_bytes + 16);
    if (rc) return rc;
    float* d_tc = static_cast<float*>(ctx->stage_in);
    uint8_t* d_tex = static_cast<uint8_t*>(ctx->stage_in) + tc_bytes;
    CK(cudaMemcpyAsync(d_tc, tex_coords, tc_bytes, cudaMemcpyHostToDevice, ctx->stream), "texture coordinates");
    CK(cudaMemcpyAsync(d_tex, texels, tex_bytes, cudaMemcpyHostToDevice, ctx->stream), "texture");
    CK(launch_render(ctx, *b, *camera, width, height, BVHGPU_ACC_TEXTURE, nullptr, shader, shader_params, nullptr,
                     d_tc, d_tex, tex_w, tex_h, static_cast<uint8_t*>(ctx->stage_out), ctx->stream),
       "render");
    CK(cudaMemcpyAsync(rgba, ctx->stage_out, 4 * px, cudaMemcpyDeviceToHost, ctx->stream), "download frame");
    rc = finish(ctx);
    if (rc) return rc;
    if (rays_traced) *rays_traced = px;
    return BVHGPU_OK;
}

// ---- scene render -----------------------------------------------------------------------------

int bvhgpu_blas_set_shading(bvhgpu_ctx* ctx, uint32_t blas_id, const float* normals, const float* tex_coords,
                            const uint8_t* texels, uint32_t tex_w, uint32_t tex_h) {
    if (!ctx) return BVHGPU_ERR_INVALID_ARG;
    DeviceBlas* b = find_blas(ctx, blas_id);
    if (!b) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown BLAS %u", blas_id);
    if (texels && (tex_w == 0 || tex_h == 0))
        return fail(ctx, BVHGPU_ERR_INVALID_ARG, "a texture needs tex_w > 0 and tex_h > 0");
    // the caller's stream may still read the old arrays
    CK(cudaStreamSynchronize(ctx->stream), "stream synchronize");
    auto replace = [&](auto** dst, const void* src, size_t bytes) -> int {
        void* p = nullptr;
        cudaError_t e = cudaMalloc(&p, std::max<size_t>(bytes, 16));
        if (e != cudaSuccess) return fail(ctx, BVHGPU_ERR_OUT_OF_MEMORY, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
        e = cudaMemcpy(p, src, bytes, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cudaFree(p);
            return cuda_fail(ctx, e, "upload shading data");
        }
        cudaFree(*dst);
        *dst = static_cast<std::remove_pointer_t<decltype(dst)>>(p);
        return BVHGPU_OK;
    };
    int rc = BVHGPU_OK;
    if (normals) rc = replace(&b->normals, normals, 36ull * b->ntris);
    if (!rc && tex_coords) rc = replace(&b->tex_coords, tex_coords, 24ull * b->ntris);
    if (!rc && texels) {
        rc = replace(&b->texels, texels, 3ull * tex_w * tex_h);
        if (!rc) {
            b->tex_w = tex_w;
            b->tex_h = tex_h;
        }
    }
    return rc;
}

int bvhgpu_render_scene(bvhgpu_ctx* ctx, uint32_t scene_id, const bvhgpu_camera* camera, int width, int height,
                        int accumulator, const float* acc_params, int shader, const float* shader_params, int lookup,
                        uint8_t* rgba, uint64_t* rays_traced) {
    if (!ctx || !camera || !rgba || width <= 0 || height <= 0) return BVHGPU_ERR_INVALID_ARG;
    if (accumulator < 0 || accumulator > 4 || shader < 0 || shader > 2)
        return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown accumulator %d or shader %d", accumulator, shader);
    if (lookup != BVHGPU_LOOKUP_REFERENCE && lookup != BVHGPU_LOOKUP_HIT_OBJECT)
        return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown lookup %d", lookup);
    if (accumulator == BVHGPU_ACC_INTERSECTION && !acc_params)
        return fail(ctx, BVHGPU_ERR_INVALID_ARG, "accumulator needs parameters");
    if ((shader == BVHGPU_SHADER_INTERSECTION || shader == BVHGPU_SHADER_DEPTH) && !shader_params)
        return fail(ctx, BVHGPU_ERR_INVALID_ARG, "shader needs parameters");
    DeviceScene* sc = find_scene(ctx, scene_id);
    if (!sc) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "unknown scene %u", scene_id);
    if (sc->nobjects == 0) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "scene %u has no objects", scene_id);
    std::vector<ShadeEntry> tab(sc->table_blas.size());
    for (size_t k = 0; k < tab.size(); ++k) {
        const DeviceBlas* b = find_blas(ctx, sc->table_blas[k]);
        if (!b) return fail(ctx, BVHGPU_ERR_INVALID_ARG, "scene %u uses a freed BLAS", scene_id);
        tab[k] = ShadeEntry{b->normals, b->tex_coords, b->texels, b->tex_w, b->tex_h, b->ntris, 0};
    }
    const size_t px = (size_t)width * height, tab_bytes = tab.size() * sizeof(ShadeEntry);
    int rc = ensure(ctx, &ctx->stage_out, &ctx->stage_out_bytes, 4 * px);
    if (!rc) rc = ensure(ctx, &ctx->stage_in, &ctx->stage_in_bytes, tab_bytes + 16);
    if (rc) return rc;
    CK(cudaMemcpyAsync(ctx->stage_in, tab.data(), tab_bytes, cudaMemcpyHostToDevice, ctx->stream), "shade table");
    CK(launch_render_scene(ctx, *sc, *camera, width, height, accumulator, acc_params, shader, shader_params,
                           static_cast<const ShadeEntry*>(ctx->stage_in), lookup,
                           static_cast<uint8_t*>(ctx->stage_out), ctx->stream),
       "render scene");
    CK(cudaMemcpyAsync(rgba, ctx->stage_out, 4 * px, cudaMemcpyDeviceToHost, ctx->stream), "download frame");
    rc = finish(ctx);
    if (rc) return rc;
    if (rays_traced) *rays_traced = px;
    return BVHGPU_OK;
}

}  // extern "C"
