// header_only_common.cuh -- host functions and page addressing shared by the
// header-only drop-in families (source/Paging.cuh, RandomWalkBasic.cuh:15-22).
// Include one family header per translation unit, as with the reference.
#pragma once
#include "pbm/dropin.cuh"

#ifndef PAGE_SIZE_DEFAULT
#define PAGE_SIZE_DEFAULT 512
#endif
#ifndef TOTAL_SIZE_GB_DEFAULT
#define TOTAL_SIZE_GB_DEFAULT 8
#endif
#ifndef GB_SIZE
#define GB_SIZE 1024ull * 1024ull * 1024ull
#endif
#ifndef TOTAL_N_PAGES_DEFAULT
#define TOTAL_N_PAGES_DEFAULT (TOTAL_SIZE_GB_DEFAULT) * (GB_SIZE) / (PAGE_SIZE_DEFAULT)
#endif
#ifndef PBM_DROPIN_SLOTS
#define PBM_DROPIN_SLOTS (1u << 24)   // per-thread cursor entries (the reference allows 10^8)
#endif

static __device__ pbm::dropin::DeviceState pbm_tu_state;   // one pool per translation unit
static pbm::dropin::HostState pbm_tu_host;
static int h_total_n_pages = 0;                            // Paging.cuh:37

/* initMemoryManagement(nGB, pageSize): RandomWalkBasic.cuh:39-48, Paging.cuh:59-85 */
__host__ inline void initMemoryManagement(int nGB = TOTAL_SIZE_GB_DEFAULT, int pageSize = PAGE_SIZE_DEFAULT) {
    pbm::dropin::DeviceState ds{};
    pbm::dropin::create_pool(pbm::dropin::gb_pages(nGB, pageSize), (uint32_t)pageSize, PBM_DROPIN_SLOTS,
                             false, &pbm_tu_host, &ds);
    h_total_n_pages = (int)pbm_tu_host.n_pages;
    cudaMemcpyToSymbol(pbm_tu_state, &ds, sizeof(ds));
#ifdef PBM_DROPIN_AFTER_INIT
    PBM_DROPIN_AFTER_INIT();   // family-specific set-up (RWMalloc.cuh: malloc tables)
#endif
}

/* pageAddress / getPageID: Paging.cuh:30-52 (one contiguous reservation) */
__device__ inline void* pageAddress(int pageID) { return pbm::page_address(pbm_tu_state.view, pageID); }
__device__ inline int getPageID(void* pageAddr) { return pbm::page_id(pbm_tu_state.view, pageAddr); }

/* getFreePagePercentage(): RandomWalkBasic_BM.cuh:117-145 */
__host__ inline float getFreePagePercentage() { return pbm::dropin::free_fraction(pbm_tu_host); }
/* resetMemoryManager(): RandomWalkBasic.cuh:86-88 */
__host__ inline void resetMemoryManager() { pbm::dropin::reset(pbm_tu_host); }
/* prefillBuffer(freePercentage): RandomWalkBasic.cuh:121-131 */
__host__ inline void prefillBuffer(float freePercentage) { pbm::dropin::prefill(pbm_tu_host, freePercentage); }
