// parallelPage_impl.cuh -- definitions of the parallelPage.cuh drop-in.
// Included by pbm/parallelPage.cuh in the header-only form (inline
// functions, state per translation unit) and compiled once into
// libpbm_dropin.a for the -rdc form (PBM_PARALLELPAGE_LIBRARY: external
// functions, one state for the whole program).
#pragma once
#include <thread>

#include "pbm/dropin.cuh"
#include "pbm/parallelPage.cuh"

#if defined(PBM_PARALLELPAGE_LIBRARY)
#define PBM_PP_DEF
#else
#define PBM_PP_DEF inline
#endif

#ifndef PBM_PP_SLOTS
#define PBM_PP_SLOTS (1u << 22)   // per-thread arms / cursors (DistClock allows 10^6 in the reference)
#endif

enum { PBM_PP_RW, PBM_PP_CRW, PBM_PP_LL, PBM_PP_SC, PBM_PP_DC, PBM_PP_CORW, PBM_PP_CORW_BM, PBM_PP_RW_BM,
       PBM_PP_CRW_BM, PBM_PP_N };

static __device__ pbm::dropin::DeviceState pbm_pp_dev[PBM_PP_N];
static pbm::dropin::HostState pbm_pp_host[PBM_PP_N];
static __device__ char* pbm_pp_pages;   // the page store shared by every strategy (pageAddress)
static char* pbm_pp_pages_host = nullptr;

// initPages*(): the strategy's own free-page map (a pool without page memory)
// and, on the first call, the page store all strategies share.
static inline void pbm_pp_init(int k, bool fifo) {
    if (!pbm_pp_pages_host) {
        const size_t bytes = (size_t)TOTAL_N_PAGES * (size_t)PAGE_SIZE;
        if (cudaMalloc(&pbm_pp_pages_host, bytes) != cudaSuccess) {
            cudaGetLastError();
            std::fprintf(stderr, "[pbm] page store of %zu bytes could not be allocated\n", bytes);
            pbm_pp_pages_host = nullptr;
            return;
        }
        cudaMemcpyToSymbol(pbm_pp_pages, &pbm_pp_pages_host, sizeof(pbm_pp_pages_host));
    }
    if (pbm_pp_host[k].pool) return;   // initialised already
    pbm::dropin::DeviceState ds{};
    // only the clustered walks and the distributed clock keep per-thread state
    const bool slots = k == PBM_PP_CRW || k == PBM_PP_DC || k == PBM_PP_CRW_BM;
    if (!pbm::dropin::create_pool(TOTAL_N_PAGES, PAGE_SIZE, slots ? PBM_PP_SLOTS : 32u, fifo, &pbm_pp_host[k], &ds,
                                  false))
        return;
    cudaMemcpyToSymbol(pbm_pp_dev, &ds, sizeof(ds), sizeof(ds) * (size_t)k);
}

static inline void pbm_pp_print(int k, const char* tag) {
    std::printf("[%s info] Number of free pages: %llu \n", tag,
                (unsigned long long)pbm::dropin::free_pages(pbm_pp_host[k]));
}

static inline void pbm_pp_reset(int k) {
    pbm::dropin::reset(pbm_pp_host[k]);
    if (k == PBM_PP_LL && pbm_pp_host[k].pool) {   // rebuild the free list of an all-free pool
        pbm_device_state d{};
        pbm_pool_device_state(pbm_pp_host[k].pool, 1, &d, nullptr);
    }
}

/* pageAddress(pageID): parallelPage.cu:15-23 */
__device__ PBM_PP_DEF void* pageAddress(int pageID) {
    return (void*)(pbm_pp_pages + (size_t)(uint32_t)pageID * PAGE_SIZE);
}

__device__ static inline int pbm_pp_tid() { return (int)pbm::dropin::global_tid(); }

/* ---- Random Walk (parallelPage.cu:111-223) ---- */
__host__ PBM_PP_DEF void initPagesRandomWalk() { pbm_pp_init(PBM_PP_RW, false); }
__device__ PBM_PP_DEF int getPageRandomWalk(int* step_count) {
    const auto& d = pbm_pp_dev[PBM_PP_RW];
    return d.valid ? pbm::walk_page(d.view, pbm::dropin::call_seed(), PBM_DROPIN_MAX_STEPS, step_count) : -1;
}
__device__ PBM_PP_DEF void freePageRandomWalk(int pageID) { pbm::dropin::free_checked(pbm_pp_dev[PBM_PP_RW], pageID); }
__host__ PBM_PP_DEF void printNumPagesLeftRandomWalk() { pbm_pp_print(PBM_PP_RW, "RW"); }
__host__ PBM_PP_DEF void resetBufferRandomWalk() { pbm_pp_reset(PBM_PP_RW); }
/* monitorBufferRandomWalk(msGap, maxCount): parallelPage.cu:209-223 -- a host
 * thread reads the occupancy every msGap ms on its own stream. */
__host__ PBM_PP_DEF void monitorBufferRandomWalk(int msGap, int maxCount) {
    pbm_pool* pool = pbm_pp_host[PBM_PP_RW].pool;
    if (!pool) return;
    std::thread([pool, msGap, maxCount]() {
        cudaStream_t s;
        if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return;
        for (int i = 0; i < maxCount; ++i) {
            uint64_t used = 0;
            if (pbm_pool_used(pool, &used, s) != PBM_OK) break;
            const uint64_t free_pages = (uint64_t)TOTAL_N_PAGES - used;
            std::printf("[RW info] Number of free pages: %llu, percentage free: %2.1f %% \n",
                        (unsigned long long)free_pages, 100.0 * (double)free_pages / TOTAL_N_PAGES);
            std::this_thread::sleep_for(std::chrono::milliseconds(msGap));
        }
        cudaStreamDestroy(s);
    }).detach();
}

/* ---- Clustered Random Walk (parallelPage.cu:231-297) ---- */
__host__ PBM_PP_DEF void initPagesClusteredRandomWalk() { pbm_pp_init(PBM_PP_CRW, false); }
__device__ PBM_PP_DEF int getPageClusteredRandomWalk(int* step_count) {
    const auto& d = pbm_pp_dev[PBM_PP_CRW];
    if (!d.valid) return -1;
    int32_t* cur = d.cursors + ((uint32_t)pbm_pp_tid() % d.max_slots);
    int32_t c = *cur;
    int id = pbm::walk_crw(d.view, &c, pbm::dropin::call_seed(), PBM_DROPIN_MAX_STEPS, step_count);
    *cur = c;
    return id;
}
__device__ PBM_PP_DEF void freePageClusteredRandomWalk(int pageID) {
    pbm::dropin::free_checked(pbm_pp_dev[PBM_PP_CRW], pageID);
}
__host__ PBM_PP_DEF void printNumPagesLeftClusteredRandomWalk() { pbm_pp_print(PBM_PP_CRW, "CRW"); }

/* ---- Linked List (parallelPage.cu:303-466): FIFO free list ---- */
__host__ PBM_PP_DEF void initPagesLinkedList() { pbm_pp_init(PBM_PP_LL, true); }
__device__ PBM_PP_DEF int getPageLinkedList(int* step_count) {
    const auto& d = pbm_pp_dev[PBM_PP_LL];
    if (!d.valid || !d.ring) return -1;
    return pbm::fifo_get(d.view, d.fifo, d.ring, d.stats, step_count);
}
__device__ PBM_PP_DEF void freePageLinkedList(int pageID, int* step_count) {
    const auto& d = pbm_pp_dev[PBM_PP_LL];
    if (step_count) *step_count = 0;
    if (d.valid && d.ring && pageID >= 0 && (uint32_t)pageID < d.view.n_pages)
        pbm::fifo_put(d.view, d.fifo, d.ring, d.stats, pageID);
}
__host__ PBM_PP_DEF void printNumPagesLeftLinkedList() { pbm_pp_print(PBM_PP_LL, "LL"); }
__host__ PBM_PP_DEF void resetBufferLinkedList() { pbm_pp_reset(PBM_PP_LL); }

/* ---- Single Clock (parallelPage.cu:471-535) ---- */
__host__ PBM_PP_DEF void initPagesSingleClock() { pbm_pp_init(PBM_PP_SC, false); }
__device__ PBM_PP_DEF int getPageSingleClock(int* step_count) {
    const auto& d = pbm_pp_dev[PBM_PP_SC];
    return d.valid ? pbm::sweep_single(d.view, d.single_arm, PBM_DROPIN_MAX_STEPS, step_count) : -1;
}
__device__ PBM_PP_DEF void freePageSingleClock(int pageID, int* step_count) {
    if (step_count) *step_count = 0;
    pbm::dropin::free_checked(pbm_pp_dev[PBM_PP_SC], pageID);
}
__host__ PBM_PP_DEF void printNumPagesLeftSingleClock() { pbm_pp_print(PBM_PP_SC, "SC"); }
__host__ PBM_PP_DEF void resetBufferSingleClock() { pbm_pp_reset(PBM_PP_SC); }

/* ---- Distributed Clock (parallelPage.cu:538-618) ---- */
__host__ PBM_PP_DEF void initPagesDistClock() { pbm_pp_init(PBM_PP_DC, false); }
__device__ PBM_PP_DEF int getPageDistClock(int* step_count) {
    const auto& d = pbm_pp_dev[PBM_PP_DC];
    if (!d.valid) return -1;
    uint32_t* arm = d.arms + ((uint32_t)pbm_pp_tid() % d.max_slots);
    uint32_t a = *arm;
    int id = pbm::sweep_dist(d.view, &a, PBM_DROPIN_MAX_STEPS, step_count);
    *arm = a;
    return id;
}
__device__ PBM_PP_DEF void freePageDistClock(int pageID, int* step_count) {
    if (step_count) *step_count = 0;
    pbm::dropin::free_checked(pbm_pp_dev[PBM_PP_DC], pageID);
}
__host__ PBM_PP_DEF void printNumPagesLeftDistClock() { pbm_pp_print(PBM_PP_DC, "DC"); }
__host__ PBM_PP_DEF void resetBufferDistClock() { pbm_pp_reset(PBM_PP_DC); }

/* ---- Collaborative Random Walk (parallelPage.cu:630-721) ---- */
__host__ PBM_PP_DEF void initPagesCollabRW() { pbm_pp_init(PBM_PP_CORW, false); }
__device__ PBM_PP_DEF int getPageCollabRW(int* step_count) {
    int s = 0;
    int id = pbm::dropin::collab_get(pbm_pp_dev[PBM_PP_CORW], &s);
    if (step_count) *step_count = s;
    return id;
}
__device__ PBM_PP_DEF void freePageCollabRW(int pageID) { pbm::dropin::free_checked(pbm_pp_dev[PBM_PP_CORW], pageID); }
__host__ PBM_PP_DEF void printNumPagesLeftCollabRW() { pbm_pp_print(PBM_PP_CORW, "CoRW"); }
__host__ PBM_PP_DEF void resetBufferCollabRW() { pbm_pp_reset(PBM_PP_CORW); }

/* ---- Collaborative Random Walk + bitmap (parallelPage.cu:733-1038) ---- */
__host__ PBM_PP_DEF void initPagesCollabRW_BM() { pbm_pp_init(PBM_PP_CORW_BM, false); }
__device__ PBM_PP_DEF int getPageCollabRW_BM(int* step_count) {
    int s = 0;
    int id = pbm::dropin::collab_get(pbm_pp_dev[PBM_PP_CORW_BM], &s);
    if (step_count) *step_count = s;
    return id;
}
/* getXPageCollabRW_BM(X): X contiguous pages (1..32) in one bitmap word */
__device__ PBM_PP_DEF int getXPageCollabRW_BM(int X, int* step_count) {
    const auto& d = pbm_pp_dev[PBM_PP_CORW_BM];
    if (!d.valid || X < 1 || X > 32) return -1;
    return pbm::walk_run(d.view, (uint32_t)X, pbm::dropin::call_seed(), PBM_DROPIN_MAX_STEPS, step_count);
}
__device__ PBM_PP_DEF void freePageCollabRW_BM(int pageID) {
    pbm::dropin::free_checked(pbm_pp_dev[PBM_PP_CORW_BM], pageID);
}
__host__ PBM_PP_DEF void printNumPagesLeftCollabRW_BM() { pbm_pp_print(PBM_PP_CORW_BM, "CoRW_BM"); }
__host__ PBM_PP_DEF void resetBufferCollabRW_BM() { pbm_pp_reset(PBM_PP_CORW_BM); }

/* ---- Random Walk + bitmap (parallelPage.cu:1042-1182) ---- */
__host__ PBM_PP_DEF void initPagesRandomWalk_BM() { pbm_pp_init(PBM_PP_RW_BM, false); }
__device__ PBM_PP_DEF int getPageRandomWalk_BM(int* step_count) {
    const auto& d = pbm_pp_dev[PBM_PP_RW_BM];
    return d.valid ? pbm::walk_word<uint32_t>(d.view, pbm::dropin::call_seed(), PBM_DROPIN_MAX_STEPS, step_count)
                   : -1;
}
__device__ PBM_PP_DEF int getXPageRandomWalk_BM(int X, int* step_count) {
    const auto& d = pbm_pp_dev[PBM_PP_RW_BM];
    if (!d.valid || X < 1 || X > 32) return -1;
    return pbm::walk_run(d.view, (uint32_t)X, pbm::dropin::call_seed(), PBM_DROPIN_MAX_STEPS, step_count);
}
__device__ PBM_PP_DEF void freePageRandomWalk_BM(int pageID) {
    pbm::dropin::free_checked(pbm_pp_dev[PBM_PP_RW_BM], pageID);
}
__host__ PBM_PP_DEF void printNumPagesLeftRandomWalk_BM() { pbm_pp_print(PBM_PP_RW_BM, "RW"); }
__host__ PBM_PP_DEF void resetBufferRandomWalk_BM() { pbm_pp_reset(PBM_PP_RW_BM); }

/* ---- Clustered Random Walk + bitmap (parallelPage.cu:1185-1320) ---- */
__host__ PBM_PP_DEF void initPagesClusteredRandomWalk_BM() { pbm_pp_init(PBM_PP_CRW_BM, false); }
__device__ PBM_PP_DEF int getPageClusteredRandomWalk_BM(int* step_count) {
    const auto& d = pbm_pp_dev[PBM_PP_CRW_BM];
    if (!d.valid) return -1;
    int32_t* cur = d.cursors + ((uint32_t)pbm_pp_tid() % d.max_slots);
    int32_t c = *cur;
    int id = pbm::walk_crw(d.view, &c, pbm::dropin::call_seed(), PBM_DROPIN_MAX_STEPS, step_count);
    *cur = c;
    return id;
}
/* declared but never defined by the reference (parallelPage.cuh:72) */
__device__ PBM_PP_DEF int getXPageClusteredRandomWalk_BM(int X, int* step_count) {
    const auto& d = pbm_pp_dev[PBM_PP_CRW_BM];
    if (!d.valid || X < 1 || X > 32) return -1;
    return pbm::walk_run(d.view, (uint32_t)X, pbm::dropin::call_seed(), PBM_DROPIN_MAX_STEPS, step_count);
}
__device__ PBM_PP_DEF void freePageClusteredRandomWalk_BM(int pageID) {
    pbm::dropin::free_checked(pbm_pp_dev[PBM_PP_CRW_BM], pageID);
}
__host__ PBM_PP_DEF void printNumPagesLeftClusteredRandomWalk_BM() { pbm_pp_print(PBM_PP_CRW_BM, "CRW_BM"); }
__host__ PBM_PP_DEF void resetBufferClusteredRandomWalk_BM() { pbm_pp_reset(PBM_PP_CRW_BM); }


__host__ PBM_PP_DEF unsigned long long pbmFreePagesLeft(int strategy) {
    if (strategy < 0 || strategy >= PBM_PP_N) return 0ull;
    return (unsigned long long)pbm::dropin::free_pages(pbm_pp_host[strategy]);
}
