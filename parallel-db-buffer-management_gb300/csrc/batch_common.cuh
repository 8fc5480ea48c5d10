// batch_common.cuh -- pieces shared by the batch kernels (pages and malloc):
// the groups' prefix sums (as a block-level routine and as a kernel), the
// group lookup, the step advance of the graph form, and the graph handle.
#pragma once
#include "internal.cuh"

namespace pbm {
namespace {

// Batches with at most this many groups keep their prefix sums in shared
// memory of every block of the persistent kernel.
constexpr uint32_t kFusedGroups = 4096;
constexpr size_t kFusedPrefixBytes = sizeof(unsigned long long) * (kFusedGroups + 1u);

// Group of request q: the g in [lo, n_groups) with prefix[g] <= q < prefix[g+1]
// (prefix in global or shared memory).
__device__ __forceinline__ uint32_t find_group_any(const unsigned long long* prefix, uint32_t n_groups,
                                                   unsigned long long q, uint32_t lo) {
    uint32_t hi = n_groups;
    while (lo + 1u < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (prefix[mid] <= q) lo = mid; else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ uint32_t find_group(const unsigned long long* prefix, uint32_t n_groups,
                                               unsigned long long q, uint32_t lo) {
    uint32_t hi = n_groups;
    while (lo + 1u < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (__ldg(prefix + mid) <= q) lo = mid; else hi = mid;
    }
    return lo;
}

// Exclusive prefix of the groups' counts into out[0..n] by the whole block
// (blockDim.x a multiple of 32, at most 1024).  Ends with a block barrier.
__device__ __forceinline__ void block_exclusive_prefix(const pbm_group* g, uint32_t n, unsigned long long* out) {
    __shared__ unsigned long long warp_tot[32];
    __shared__ unsigned long long carry;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (uint32_t base = 0; base < n; base += blockDim.x) {
        uint32_t i = base + threadIdx.x;
        unsigned long long c = i < n ? (unsigned long long)g[i].count : 0ull;
        unsigned long long incl = c;
        for (int d = 1; d < 32; d <<= 1) {
            unsigned long long y = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= d) incl += y;
        }
        if (lane == 31) warp_tot[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            unsigned long long t = lane < nwarps ? warp_tot[lane] : 0ull;
            unsigned long long ti = t;
            for (int d = 1; d < 32; d <<= 1) {
                unsigned long long y = __shfl_up_sync(0xffffffffu, ti, d);
                if (lane >= d) ti += y;
            }
            if (lane < nwarps) warp_tot[lane] = ti - t;   // exclusive warp offsets
        }
        __syncthreads();
        unsigned long long excl = carry + warp_tot[warp] + incl - c;
        if (i < n) out[i] = excl;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = excl + c;
        __syncthreads();
    }
    if (threadIdx.x == 0) out[n] = carry;
    __syncthreads();
}

// Exclusive prefix of one step's groups (one block of 1024 threads).
// Graph forms keep a monotone replay counter -- in device memory (d_step) or
// in the launch's parameters (step, when d_step is null); replay k reads
// descriptor table k mod n_steps (so a graph may be replayed any number of
// times).
__global__ void k_batch_prefix(const pbm_group* groups, uint32_t n_groups, const uint32_t* d_step,
                               uint32_t step, uint32_t n_steps, unsigned long long* prefix) {
    const uint32_t k = (d_step ? *d_step : step) % (n_steps ? n_steps : 1u);
    block_exclusive_prefix(groups + (size_t)k * n_groups, n_groups, prefix);
}

__global__ void k_step_advance(uint32_t* d_step) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *d_step += 1u;
}

}  // namespace
}  // namespace pbm

// A captured graph.  Its replay counter lives either in device memory
// (d_step, advanced by a kernel of the graph) or on the host (host_step,
// written into the kernels' parameters before each replay: the launches
// then read the step with their parameters instead of from memory).
struct pbm_graph {
    cudaGraph_t graph;
    cudaGraphExec_t exec;
    uint32_t* d_step;                 // device replay counter (null: host_step)
    uint32_t host_step;
    unsigned long long* d_pools;      // the batch kernel's tail-pool counters (may be null)
    unsigned long long* d_prefix;
    unsigned long long launches_per_replay;
    int device;                       // the pool's device: replays run there
    // host-counted form: the kernel nodes whose parameters carry the step,
    // their launch settings, and the parameter values they were captured with
    cudaGraphNode_t batch_node, prefix_node;
    cudaKernelNodeParams batch_kp, prefix_kp;
    alignas(16) unsigned char batch_args[256];
    const pbm_group* prefix_groups;
    uint32_t prefix_n_groups, prefix_n_steps;
    unsigned long long* prefix_out;
};
