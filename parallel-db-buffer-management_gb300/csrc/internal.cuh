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
}  // namespace pbm
