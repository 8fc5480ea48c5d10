// internal.cuh -- host/device internals shared by the libpbm translation units.
#pragma once
#include <cuda_runtime.h>
#include <atomic>
#include <cstdint>
#include <cstdio>

#include "pbm.h"
#include "pbm/pbm_device.cuh"

namespace pbm {

// Invariant-check counters.
struct CheckCounters {
    unsigned long long ok, failed, out_of_range, duplicates, not_marked, used;
};

extern std::atomic<unsigned long long> g_launches;
inline void count_launch(unsigned long long n = 1) { g_launches.fetch_add(n, std::memory_order_relaxed); }

int sm_count();
bool device_writable(const void* p);

constexpr uint32_t kDefaultMaxSteps = 4096;

// Adds every thread's N counters to dst[0..N) with one global atomic per
// counter per block: warp shuffles, then one shared atomic per warp.  Every
// thread of the block calls it (after its loop, converged); blocks whose size
// is not a multiple of 32 (one-thread replays) add directly.  Per-thread
// atomics on a shared counter would serialise on one L2 address (~1.5 G/s).
template <int N>
__device__ __forceinline__ void block_add_counters(const unsigned long long (&v)[N],
                                                   unsigned long long* const (&dst)[N]) {
    if (blockDim.x & 31u) {
        for (int k = 0; k < N; ++k)
            if (v[k]) atomicAdd(dst[k], v[k]);
        return;
    }
    __shared__ unsigned long long sh[N];
    __syncthreads();   // an earlier call in the same kernel may still read sh
    if (threadIdx.x < (unsigned)N) sh[threadIdx.x] = 0ull;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < N; ++k) {
        unsigned long long x = v[k];
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) x += __shfl_down_sync(0xffffffffu, x, d);
        if ((threadIdx.x & 31u) == 0u && x) atomicAdd(&sh[k], x);
    }
    __syncthreads();
    if (threadIdx.x < (unsigned)N && sh[threadIdx.x]) atomicAdd(dst[threadIdx.x], sh[threadIdx.x]);
}
// Makes a device current for the rest of the calling scope and restores the
// caller's device when the scope ends.  Every entry point that takes a pool
// (or an object built on one) opens one with the pool's device, so a process
// may hold one pool per GPU and call into any of them from any current
// device.  A negative ordinal (no pool) switches nothing.
struct DeviceScope {
    int prev = -1;
    bool switched = false;
    explicit DeviceScope(int dev) {
        if (dev >= 0 && cudaGetDevice(&prev) == cudaSuccess && prev != dev && cudaSetDevice(dev) == cudaSuccess)
            switched = true;
    }
    ~DeviceScope() {
        if (switched) cudaSetDevice(prev);
    }
    DeviceScope(const DeviceScope&) = delete;
    DeviceScope& operator=(const DeviceScope&) = delete;
};

constexpr int kDefaultBlock = 256;
constexpr int kCappedBlocks = 5;   // resident blocks the register-capped batch kernels are built for

}  // namespace pbm

struct pbm_pool {
    pbm::PoolView view;
    uint64_t n_pages;
    uint32_t page_size;
    uint32_t flags;
    uint32_t max_slots;
    size_t bitmap_bytes;            // n_words32 (even) * 4
    uint64_t padding_bits;          // set bits past n_pages
    uint32_t* d_words;
    char* d_base;
    pbm::DevStats* d_stats;
    int32_t* d_cursors;             // clustered walk, per slot
    uint32_t* d_arms;               // distributed clock, per slot
    unsigned long long* d_arm;      // single clock
    int32_t* d_ring;                // FIFO ring, n_pages entries (lazily built)
    pbm::FifoState* d_fifo;
    bool fifo_valid;
    uint32_t* d_seen;               // check scratch: one bit per page
    pbm::CheckCounters* d_check;
    unsigned long long* d_scan;     // scratch for prefix sums (per-block partials)
    unsigned long long* d_prefix;   // batch prefix (n_groups + 1)
    pbm::LaunchBudget* d_budget;    // fail-fast launch budget: free pages at launch start
    int32_t* d_free_list;           // the budget pass's list of free pages (list mode)
    uint64_t free_list_cap;
    unsigned long long* d_budget_blocks;   // free pages per block slice of the budget pass
    uint32_t budget_blocks;
    uint32_t prefix_cap;
    int device;
};

#define PBM_CUDA_TRY(expr)                                                          \
    do {                                                                            \
        cudaError_t _e = (expr);                                                    \
        if (_e != cudaSuccess) {                                                    \
            std::fprintf(stderr, "[pbm] %s failed: %s (%s:%d)\n", #expr,           \
                         cudaGetErrorString(_e), __FILE__, __LINE__);               \
            cudaGetLastError(); /* do not leave the error for the next caller */   \
            return PBM_ERR_CUDA;                                                    \
        }                                                                           \
    } while (0)

#define PBM_ON_POOL_DEVICE(pool) pbm::DeviceScope pbm_device_scope_((pool) ? (pool)->device : -1)

#define PBM_LAUNCH_CHECK()                                                          \
    do {                                                                            \
        cudaError_t _e = cudaGetLastError();                                        \
        if (_e != cudaSuccess) {                                                    \
            std::fprintf(stderr, "[pbm] launch failed: %s (%s:%d)\n",              \
                         cudaGetErrorString(_e), __FILE__, __LINE__);               \
            return PBM_ERR_CUDA;                                                    \
        }                                                                           \
        pbm::count_launch();                                                        \
    } while (0)

namespace pbm {
// Implemented in pool.cu
int fifo_build(pbm_pool* pool, cudaStream_t s);
int popcount_used(pbm_pool* pool, uint64_t* used, cudaStream_t s);
// Counts the pool's free pages into pool->d_budget on stream s (no sync); a
// launch of n_requests that asks for at least half of them also gets them
// listed in order in pool->d_free_list (list mode, when they fit).
int budget_prepare(pbm_pool* pool, uint64_t n_requests, cudaStream_t s);
}  // namespace pbm
