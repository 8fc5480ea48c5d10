// Drop-in for source/RWMalloc.cuh: collaborative getPage, n-page runs
// (getNPage) and the warp-coalescing mallocRW / freeRW, over a pool set up by
// initMemoryManagement.  mallocRW rounds each request up to a power-of-two
// size class (16 B .. 64 KiB); the calling lanes' sub-page requests share one
// run and the last freeRW of a run releases it.  The page size must be a
// power of two between 2 KiB and 64 KiB (the reference needs at least 2 KiB
// for 64 KiB requests as well).
#pragma once
static inline void pbm_rwmalloc_after_init();
#define PBM_DROPIN_AFTER_INIT pbm_rwmalloc_after_init
#include "pbm/header_only_common.cuh"
#include "pbm/pbm_malloc.cuh"

static __device__ pbm::MallocView pbm_tu_malloc;

/* getPage(int* stepCount): RWMalloc.cuh:113-149 (collaborative, as in the reference) */
__device__ inline int getPage(int* stepCount = 0) {
    int s = 0;
    int id = pbm::dropin::collab_get(pbm_tu_state, &s);
    if (stepCount) *stepCount = s;
    return id;
}

/* getNPage(n, stepCount): RWMalloc.cuh:203-248 -- n contiguous pages (1..32)
 * inside one bitmap word; n == 0 returns 0 as in the reference. */
__device__ inline int getNPage(int n, int* stepCount = 0) {
    if (n <= 0) { if (stepCount) *stepCount = 0; return 0; }
    if (!pbm_tu_state.valid || n > 32) return -1;
    return pbm::walk_run(pbm_tu_state.view, (uint32_t)n, pbm::dropin::call_seed(), PBM_DROPIN_MAX_STEPS, stepCount);
}

__device__ inline void* getPagePtr() {
    int id = getPage();
    return id >= 0 ? pageAddress(id) : nullptr;
}

/* freePage(pageID): RWMalloc.cuh:72-76 */
__device__ inline void freePage(int pageID) { pbm::dropin::free_checked(pbm_tu_state, pageID); }

/* mallocRW(size): RWMalloc.cuh:299-326.  Every calling lane gets its own
 * block (nullptr on failure); the calling lanes must be converged. */
__device__ inline void* mallocRW(size_t size) {
    const uint32_t active = __activemask();
    const int32_t own = pbm::dropin::call_seed();
    const int32_t shared = __shfl_sync(active, own, __ffs((int)active) - 1) ^ 0x5bd1e995;
    return pbm::malloc_group(pbm_tu_malloc, active, (uint64_t)size, shared & 0x7fffffff, own,
                             PBM_DROPIN_MAX_STEPS, false, nullptr);
}

/* freeRW(ptr): RWMalloc.cuh:329-334 (the calling lanes must be converged) */
__device__ inline void freeRW(void* ptr) { pbm::free_group(pbm_tu_malloc, __activemask(), ptr); }

/* initMemoryManagement (header_only_common.cuh) calls this: malloc side
 * tables for the pool and their device view for mallocRW / freeRW. */
static inline void pbm_rwmalloc_after_init() {
    if (!pbm_tu_host.pool) return;
    if (pbm_malloc_init(pbm_tu_host.pool) != PBM_OK) {
        std::fprintf(stderr, "[pbm] mallocRW needs a power-of-two page size of 2 KiB .. 64 KiB\n");
        return;
    }
    pbm_device_state d{};
    pbm::MallocView mv{};
    if (pbm_pool_device_state(pbm_tu_host.pool, 0, &d, nullptr) != PBM_OK ||
        pbm_malloc_tables(pbm_tu_host.pool, (void**)&mv.start_of, (void**)&mv.live, (void**)&mv.len_of) != PBM_OK)
        return;
    mv.pool.words = (uint32_t*)d.words;
    mv.pool.base = (char*)d.base;
    mv.pool.n_pages = (uint32_t)d.n_pages;
    mv.pool.n_words32 = d.n_words32;
    mv.pool.n_words64 = d.n_words64;
    mv.pool.page_size = d.page_size;
    uint32_t sh = 0;
    while ((1u << sh) < d.page_size) ++sh;
    mv.page_shift = sh;
    cudaMemcpyToSymbol(pbm_tu_malloc, &mv, sizeof(mv));
}
