// dropin.cuh -- shared plumbing of the drop-in headers (RandomWalkBasic.cuh,
// RandomWalkBasic_BM.cuh, CollabRW_BM.cuh, CRW_BM.cuh, RWMalloc.cuh,
// parallelPage.cuh, malloc.cuh).
//
// The reference keeps one pool per translation unit in __device__ globals
// written with cudaMemcpyToSymbol (source/Paging.cuh:37-42, 69-81).  The
// drop-in headers do the same with a pool of libpbm.so: the host init
// function creates the pool and copies its device descriptor into a
// __device__ variable of the including translation unit, which the device
// functions read.  Link the caller with -lpbm.
//
// Differences from the reference, by design: walks are bounded
// (PBM_DROPIN_MAX_STEPS random jumps) and return -1 instead of trapping or
// spinning; host errors are reported on stderr and leave the pool unset
// (device calls then return -1) instead of calling exit().
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>

#include "pbm.h"
#include "pbm/pbm_device.cuh"

#ifndef PBM_DROPIN_MAX_STEPS
#define PBM_DROPIN_MAX_STEPS 65536u
#endif

namespace pbm {
namespace dropin {

// Everything the device side of a drop-in family reads.
struct DeviceState {
    PoolView view;
    int32_t* cursors;
    uint32_t* arms;
    unsigned long long* single_arm;
    FifoState* fifo;
    int32_t* ring;
    DevStats* stats;
    uint32_t max_slots;
    uint32_t valid;
};

struct HostState {
    pbm_pool* pool = nullptr;
    uint64_t n_pages = 0;
};

inline bool create_pool(uint64_t n_pages, uint32_t page_size, uint32_t max_slots, bool build_fifo,
                        HostState* hs, DeviceState* ds, bool with_pages = true) {
    pbm_pool_config c{};
    c.n_pages = n_pages;
    c.page_size = page_size;
    c.flags = with_pages ? PBM_POOL_MATERIALIZE : 0u;
    c.max_slots = max_slots;
    int rc = pbm_pool_create(&c, &hs->pool);
    if (rc != PBM_OK) {
        std::fprintf(stderr, "[pbm] pool of %llu pages x %u B could not be created (status %d)\n",
                     (unsigned long long)n_pages, page_size, rc);
        hs->pool = nullptr;
        *ds = DeviceState{};
        return false;
    }
    pbm_device_state d{};
    rc = pbm_pool_device_state(hs->pool, build_fifo ? 1 : 0, &d, nullptr);
    if (rc != PBM_OK) {
        std::fprintf(stderr, "[pbm] pool state unavailable (status %d)\n", rc);
        return false;
    }
    hs->n_pages = n_pages;
    ds->view.words = (uint32_t*)d.words;
    ds->view.base = (char*)d.base;
    ds->view.n_pages = (uint32_t)d.n_pages;
    ds->view.n_words32 = d.n_words32;
    ds->view.n_words64 = d.n_words64;
    ds->view.page_size = d.page_size;
    ds->cursors = (int32_t*)d.cursors;
    ds->arms = (uint32_t*)d.arms;
    ds->single_arm = (unsigned long long*)d.single_arm;
    ds->fifo = (FifoState*)d.fifo_state;
    ds->ring = (int32_t*)d.fifo_ring;
    ds->stats = (DevStats*)d.stats;
    ds->max_slots = d.max_slots;
    ds->valid = 1;
    return true;
}

inline uint64_t gb_pages(int nGB, int pageSize) {
    return (uint64_t)nGB * (1ull << 30) / (uint64_t)(pageSize > 0 ? pageSize : 1);
}

inline float free_fraction(const HostState& hs) {
    if (!hs.pool) return 0.f;
    uint64_t used = 0;
    if (pbm_pool_used(hs.pool, &used, nullptr) != PBM_OK) return 0.f;
    return (float)(hs.n_pages - used) / (float)hs.n_pages;
}

inline uint64_t free_pages(const HostState& hs) {
    if (!hs.pool) return 0;
    uint64_t used = 0;
    pbm_pool_used(hs.pool, &used, nullptr);
    return hs.n_pages - used;
}

inline void reset(HostState& hs) {
    if (hs.pool) pbm_pool_reset(hs.pool, nullptr);
    cudaDeviceSynchronize();
}

// prefillBuffer(freePercentage): an allocation run of (1 - f) * T pages
// (RandomWalkBasic.cuh:121-131), with the collaborative walk.
inline void prefill(HostState& hs, float freePercentage) {
    if (!hs.pool) return;
    uint64_t n = (uint64_t)((1.0f - freePercentage) * (float)hs.n_pages);
    if (n == 0) return;
    int32_t* ids = nullptr;
    if (cudaMalloc(&ids, n * sizeof(int32_t)) != cudaSuccess) { cudaGetLastError(); return; }
    pbm_walk_config c{};
    c.strategy = PBM_COLLAB_RW_BM;
    c.word_bits = 32;
    c.collab_width = 32;
    c.max_steps = 1u << 16;
    pbm_alloc(hs.pool, &c, (uint32_t)n, 0x5eedu, ids, nullptr, nullptr);
    cudaDeviceSynchronize();
    cudaFree(ids);
}

__device__ __forceinline__ uint32_t global_tid() {
    const uint32_t block = (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
    const uint32_t in_block = (threadIdx.z * blockDim.y + threadIdx.y) * blockDim.x + threadIdx.x;
    return block * (blockDim.x * blockDim.y * blockDim.z) + in_block;
}

// Per-call seed: the reference mixes the thread id with clock()
// (RandomWalkBasic.cuh:55-57); here both go through request_seed.
__device__ __forceinline__ int32_t call_seed() {
    return request_seed((uint32_t)clock64(), global_tid());
}

// Per-warp scratch of the collaborative walks (32 ints per warp of a 1-D block
// of at most 1024 threads, like the reference's S_pageIDs_block[1024]).
__device__ __forceinline__ volatile int32_t* warp_slots() {
    __shared__ int32_t pbm_dropin_slots[1024];
    return pbm_dropin_slots + (threadIdx.x & ~31u);
}

__device__ __forceinline__ int32_t collab_get(const DeviceState& d, int32_t* steps) {
    if (!d.valid) return -1;
    const uint32_t active = __activemask();
    const int32_t seed = __shfl_sync(active, call_seed(), __ffs((int)active) - 1);
    return walk_collab_masked<uint32_t>(d.view, active, true, seed, PBM_DROPIN_MAX_STEPS, warp_slots(), steps);
}

__device__ __forceinline__ void free_checked(const DeviceState& d, int pageID) {
    if (d.valid && pageID >= 0 && (uint32_t)pageID < d.view.n_pages) free_page(d.view, pageID);
}

}  // namespace dropin
}  // namespace pbm
