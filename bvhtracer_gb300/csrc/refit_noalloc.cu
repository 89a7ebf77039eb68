// Allocation-free BVH refit: bvhgpu_refit_noalloc (see include/bvhgpu.h).
//
// Some callers of this library cannot call cudaMalloc at all: engines that reserve every byte
// of device memory up front in their own pool and forbid further driver allocations, and
// latency-critical threads on which a driver allocation (which can synchronise the device)
// is not allowed.  This entry point refits a node array the caller already owns, in the
// reference's 32-byte layout, against triangles the caller owns, and allocates nothing: its
// scratch memory (parent links and arrival counters) is the fixed-size device array below,
// which every GPU that loads the library holds until the process exits.
//
// Results are the same as bvhgpu_blas_refit (Bvh::refit, bvh.rs:469-493): leaves fold their
// triangles' vertices in index order, a branch takes min/max of (left, right) in that order,
// node 1 (the unused filler) is never touched.
#include <cuda_runtime.h>

#include <cfloat>
#include <cstdint>
#include <mutex>

#include "../../include/bvhgpu.h"

namespace {

constexpr uint32_t kNone = 0xFFFFFFFFu;

// Scratch: parent link and arrival counter per node (2 x 4 bytes x BVHGPU_NOALLOC_MAX_NODES = 8 MiB).
static __device__ __align__(256) uint32_t g_refit_scratch[2u * BVHGPU_NOALLOC_MAX_NODES];

// Device address of g_refit_scratch per device, looked up once with that device current (the
// first call on the device).  cudaDeviceReset destroys the context that address belongs to, so a
// process that resets a device must not call bvhgpu_refit_noalloc on that device afterwards.
constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
uint32_t* g_scratch_addr[kMaxDevices] = {};

int scratch_for_current_device(uint32_t** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return BVHGPU_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_refit_scratch);
        if (e != cudaSuccess || p == nullptr) return BVHGPU_ERR_CUDA;
        g_scratch_addr[dev] = static_cast<uint32_t*>(p);
    }
    *out = g_scratch_addr[dev];
    return BVHGPU_OK;
}

// f32::min / f32::max with the first operand kept on equality (same rule as the other kernels).
__device__ __forceinline__ float min_ni(float a, float b) {
    if (a != a) return b;
    if (b != b) return a;
    return (b < a) ? b : a;
}
__device__ __forceinline__ float max_ni(float a, float b) {
    if (a != a) return b;
    if (b != b) return a;
    return (b > a) ? b : a;
}

// Status values OR-ed into the caller's *status word for malformed node arrays.
constexpr uint32_t kBadChild = 1u;     // a branch's child index is out of range or not above it
constexpr uint32_t kBadLeaf = 2u;      // a leaf addresses triangles past ntris
constexpr uint32_t kSharedChild = 4u;  // a node claimed as a child by two branches

// Parent links of every branch's two children.  Indices are checked before any access; a
// malformed branch is skipped and reported in *status.  A child index is always above its
// parent's, so the bottom-up walk below only moves to lower indices and ends.
__global__ void k_links(const bvhgpu_node* __restrict__ nodes, uint32_t nodes_used, uint32_t* parent,
                        uint32_t* status) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nodes_used || i == 1u) return;
    const bvhgpu_node n = nodes[i];
    if (n.primitive_count != 0u) return;
    uint32_t l = n.left_first;
    if (l <= i || l < 2u || (uint64_t)l + 1u >= nodes_used) {
        if (status) atomicOr(status, kBadChild);
        return;
    }
    // first claim wins; a second branch claiming the same child is reported (and, missing an
    // arrival, never computed)
    const uint32_t a = atomicCAS(&parent[l], kNone, i);
    const uint32_t b = atomicCAS(&parent[l + 1u], kNone, i);
    if ((a != kNone || b != kNone) && status) atomicOr(status, kSharedChild);
}

// Bottom-up refit: one thread per leaf; the second child to arrive at a parent computes it.
__global__ void k_refit_nodes(bvhgpu_node* nodes, uint32_t nodes_used, const float* __restrict__ tris,
                              uint32_t ntris, const uint32_t* __restrict__ parent, uint32_t* counters,
                              uint32_t* status) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nodes_used || i == 1u) return;
    const uint32_t cnt = nodes[i].primitive_count;
    if (cnt == 0u) return;
    const uint32_t first = nodes[i].left_first;
    if ((uint64_t)first + cnt > ntris) {
        if (status) atomicOr(status, kBadLeaf);
        return;
    }
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
    float hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (uint32_t k = 0; k < cnt; ++k) {  // update_node_bounds (bvh.rs:317-330)
        const float* t = tris + 9ull * (first + k);
        for (int c = 0; c < 3; ++c) {
            lo[c] = min_ni(min_ni(min_ni(lo[c], t[c]), t[3 + c]), t[6 + c]);
            hi[c] = max_ni(max_ni(max_ni(hi[c], t[c]), t[3 + c]), t[6 + c]);
        }
    }
    for (int c = 0; c < 3; ++c) {
        nodes[i].bounds_min[c] = lo[c];
        nodes[i].bounds_max[c] = hi[c];
    }
    __threadfence();
    uint32_t p = parent[i];
    while (p != kNone) {
        if (atomicAdd(&counters[p], 1u) == 0u) return;  // the sibling is not done yet
        counters[p] = 0u;
        __threadfence();
        const uint32_t l = nodes[p].left_first;
        for (int c = 0; c < 3; ++c) {  // bvh.rs:490-491
            float lmin = __ldcg(&nodes[l].bounds_min[c]), rmin = __ldcg(&nodes[l + 1u].bounds_min[c]);
            float lmax = __ldcg(&nodes[l].bounds_max[c]), rmax = __ldcg(&nodes[l + 1u].bounds_max[c]);
            __stcg(&nodes[p].bounds_min[c], min_ni(lmin, rmin));
            __stcg(&nodes[p].bounds_max[c], max_ni(lmax, rmax));
        }
        __threadfence();
        p = parent[p];
    }
}

}  // namespace

extern "C" int bvhgpu_refit_noalloc(bvhgpu_node* d_nodes, uint32_t nodes_used, const bvhgpu_triangle* d_tris,
                                    uint32_t ntris, bvhgpu_stream stream, uint32_t* d_status) {
    if (!d_nodes || !d_tris || nodes_used == 0 || ntris == 0) return BVHGPU_ERR_INVALID_ARG;
    if (nodes_used > BVHGPU_NOALLOC_MAX_NODES) return BVHGPU_ERR_TOO_LARGE;
    uint32_t* scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    uint32_t* parent = scratch;
    uint32_t* counters = scratch + BVHGPU_NOALLOC_MAX_NODES;
    // The scratch keeps the previous call's contents: parent links restart at "none", counters at 0.
    if (cudaMemsetAsync(parent, 0xFF, 4ull * nodes_used, s) != cudaSuccess ||
        cudaMemsetAsync(counters, 0, 4ull * nodes_used, s) != cudaSuccess)
        return BVHGPU_ERR_CUDA;
    // launch errors are read with cudaPeekAtLastError, which leaves the runtime's error state as
    // it is for the caller's own error handling
    const unsigned grid = (nodes_used + 127u) / 128u;
    k_links<<<grid, 128, 0, s>>>(d_nodes, nodes_used, parent, d_status);
    if (cudaPeekAtLastError() != cudaSuccess) return BVHGPU_ERR_CUDA;
    k_refit_nodes<<<grid, 128, 0, s>>>(d_nodes, nodes_used, reinterpret_cast<const float*>(d_tris), ntris, parent,
                                       counters, d_status);
    return cudaPeekAtLastError() == cudaSuccess ? BVHGPU_OK : BVHGPU_ERR_CUDA;
}
