// Drop-in for source/parallelPage.cuh + parallelPage.cu: the nine suffixed
// strategies of the monolithic API, each with its own pool of TOTAL_N_PAGES
// pages of PAGE_SIZE bytes (compile-time, as in the reference; override the
// macros before including).  Header-only: each translation unit that includes
// it has its own pools (the reference shares one set across translation
// units through -rdc).  Every walk is bounded (PBM_DROPIN_MAX_STEPS) and
// returns -1 instead of trapping; int-per-page maps are bitmaps here.
#pragma once
#include <thread>

#include "pbm/dropin.cuh"

#ifndef TOTAL_N_PAGES
#define TOTAL_N_PAGES 41900000
#endif
#ifndef PAGE_SIZE
#define PAGE_SIZE 264
#endif
#ifndef PBM_PP_SLOTS
#define PBM_PP_SLOTS (1u << 22)   // per-thread arms / cursors (DistClock allows 10^6 in the reference)
#endif

enum { PBM_PP_RW, PBM_PP_CRW, PBM_PP_LL, PBM_PP_SC, PBM_PP_DC, PBM_PP_CORW, PBM_PP_CORW_BM, PBM_PP_RW_BM,
       PBM_PP_CRW_BM, PBM_PP_N };

static __device__ pbm::dropin::DeviceState pbm_pp_dev[PBM_PP_N];
static pbm::dropin::HostState pbm_pp_host[PBM_PP_N];
static __device__ void* pbm_pp_base;   // page memory of the last pool initialised (pageAddress)

static inline void pbm_pp_init(int k, bool fifo) {
    pbm::dropin::DeviceState ds{};
    if (!pbm::dropin::create_pool(TOTAL_N_PAGES, PAGE_SIZE, PBM_PP_SLOTS, fifo, &pbm_pp_host[k], &ds)) return;
    cudaMemcpyToSymbol(pbm_pp_dev, &ds, sizeof(ds), sizeof(ds) * (size_t)k);
    void* base = ds.view.base;
    cudaMemcpyToSymbol(pbm_pp_base, &base, sizeof(base));
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
__device__ inline void* pageAddress(int pageID) {
    return (void*)((char*)pbm_pp_base + (size_t)(uint32_t)pageID * PAGE_SIZE);
}

__device__ inline int pbm_pp_tid() { return (int)pbm::dropin::global_tid(); }

/* ---- Random Walk (parallelPage.cu:111-223) ---- */
__host__ inline void initPagesRandomWalk() { pbm_pp_init(PBM_PP_RW, false); }
__device__ inline int getPageRandomWalk(int* step_count = 0) {
    const auto& d = pbm_pp_dev[PBM_PP_RW];
    return d.valid ? pbm::walk_page(d.view, pbm::dropin::call_seed(), PBM_DROPIN_MAX_STEPS, step_count) : -1;
}
__device__ inline void freePageRandomWalk(int pageID) { pbm::dropin::free_checked(pbm_pp_dev[PBM_PP_RW], pageID); }
__host__ inline void printNumPagesLeftRandomWalk() { pbm_pp_print(PBM_PP_RW, "RW"); }
__host__ inline void resetBufferRandomWalk() { pbm_pp_reset(PBM_PP_RW); }
/* monitorBufferRandomWalk(msGap, maxCount): parallelPage.cu:209-223 -- a host
 * thread reads the occupancy every msGap ms on its own stream. */
__host__ inline void monitorBufferRandomWalk(int msGap = 100, int maxCount = 100) {
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
__host__ inline void initPagesClusteredRandomWalk() { pbm_pp_init(PBM_PP_CRW, false); }
__device__ inline int getPageClusteredRandomWalk(int* step_count = 0) {
    const auto& d = pbm_pp_dev[PBM_PP_CRW];
    if (!d.valid) return -1;
    int32_t* cur = d.cursors + ((uint32_t)pbm_pp_tid() % d.max_slots);
    int32_t c = *cur;
    int id = pbm::walk_crw(d.view, &c, pbm::dropin::call_seed(), PBM_DROPIN_MAX_STEPS, step_count);
    *cur = c;
    return id;
}
__device__ inline void freePageClusteredRandomWalk(int pageID) {
    pbm::dropin::free_checked(pbm_pp_dev[PBM_PP_CRW], pageID);
}
__host__ inline void printNumPagesLeftClusteredRandomWalk() { pbm_pp_print(PBM_PP_CRW, "CRW"); }

/* ---- Linked List (parallelPage.cu:303-466): FIFO free list ---- */
__host__ inline void initPagesLinkedList() { pbm_pp_init(PBM_PP_LL, true); }
__device__ inline int getPageLinkedList(int* step_count = 0) {
    const auto& d = pbm_pp_dev[PBM_PP_LL];
    if (!d.valid || !d.ring) return -1;
    return pbm::fifo_get(d.view, d.fifo, d.ring, d.stats, step_count);
}
__device__ inline void freePageLinkedList(int pageID, int* step_count = 0) {
    const auto& d = pbm_pp_dev[PBM_PP_LL];
    if (step_count) *step_count = 0;
    if (d.valid && d.ring && pageID >= 0 && (uint32_t)pageID < d.view.n_pages)
        pbm::fifo_put(d.view, d.fifo, d.ring, d.stats, pageID);
}
__host__ inline void printNumPagesLeftLinkedList() { pbm_pp_print(PBM_PP_LL, "LL"); }
__host__ inline void resetBufferLinkedList() { pbm_pp_reset(PBM_PP_LL); }

/* ---- Single Clock (parallelPage.cu:471-535) ---- */
__host__ inline void initPagesSingleClock() { pbm_pp_init(PBM_PP_SC, false); }
__device__ inline int getPageSingleClock(int* step_count = 0) {
    const auto& d = pbm_pp_dev[PBM_PP_SC];
    return d.valid ? pbm::sweep_single(d.view, d.single_arm, PBM_DROPIN_MAX_STEPS, step_count) : -1;
}
__device__ inline void freePageSingleClock(int pageID, int* step_count = 0) {
    if (step_count) *step_count = 0;
    pbm::dropin::free_checked(pbm_pp_dev[PBM_PP_SC], pageID);
}
__host__ inline void printNumPagesLeftSingleClock() { pbm_pp_print(PBM_PP_SC, "SC"); }
__host__ inline void resetBufferSingleClock() { pbm_pp_reset(PBM_PP_SC); }

/* ---- Distributed Clock (parallelPage.cu:538-618) ---- */
__host__ inline void initPagesDistClock() { pbm_pp_init(PBM_PP_DC, false); }
__device__ inline int getPageDistClock(int* step_count = 0) {
    const auto& d = pbm_pp_dev[PBM_PP_DC];
    if (!d.valid) return -1;
    uint32_t* arm = d.arms + ((uint32_t)pbm_pp_tid() % d.max_slots);
    uint32_t a = *arm;
    int id = pbm::sweep_dist(d.view, &a, PBM_DROPIN_MAX_STEPS, step_count);
    *arm = a;
    return id;
}
__device__ inline void freePageDistClock(int pageID, int* step_count = 0) {
    if (step_count) *step_count = 0;
    pbm::dropin::free_checked(pbm_pp_dev[PBM_PP_DC], pageID);
}
__host__ inline void printNumPagesLeftDistClock() { pbm_pp_print(PBM_PP_DC, "DC"); }
__host__ inline void resetBufferDistClock() { pbm_pp_reset(PBM_PP_DC); }

/* ---- Collaborative Random Walk (parallelPage.cu:630-721) ---- */
__host__ inline void initPagesCollabRW() { pbm_pp_init(PBM_PP_CORW, false); }
__device__ inline int getPageCollabRW(int* step_count = 0) {
    int s = 0;
    int id = pbm::dropin::collab_get(pbm_pp_dev[PBM_PP_CORW], &s);
    if (step_count) *step_count = s;
    return id;
}
__device__ inline void freePageCollabRW(int pageID) { pbm::dropin::free_checked(pbm_pp_dev[PBM_PP_CORW], pageID); }
__host__ inline void printNumPagesLeftCollabRW() { pbm_pp_print(PBM_PP_CORW, "CoRW"); }
__host__ inline void resetBufferCollabRW() { pbm_pp_reset(PBM_PP_CORW); }

/* ---- Collaborative Random Walk + bitmap (parallelPage.cu:733-1038) ---- */
__host__ inline void initPagesCollabRW_BM() { pbm_pp_init(PBM_PP_CORW_BM, false); }
__device__ inline int getPageCollabRW_BM(int* step_count = 0) {
    int s = 0;
    int id = pbm::dropin::collab_get(pbm_pp_dev[PBM_PP_CORW_BM], &s);
    if (step_count) *step_count = s;
    return id;
}
/* getXPageCollabRW_BM(X): X contiguous pages (1..32) in one bitmap word */
__device__ inline int getXPageCollabRW_BM(int X, int* step_count = 0) {
    const auto& d = pbm_pp_dev[PBM_PP_CORW_BM];
    if (!d.valid || X < 1 || X > 32) return -1;
    return pbm::walk_run(d.view, (uint32_t)X, pbm::dropin::call_seed(), PBM_DROPIN_MAX_STEPS, step_count);
}
__device__ inline void freePageCollabRW_BM(int pageID) {
    pbm::dropin::free_checked(pbm_pp_dev[PBM_PP_CORW_BM], pageID);
}
__host__ inline void printNumPagesLeftCollabRW_BM() { pbm_pp_print(PBM_PP_CORW_BM, "CoRW_BM"); }
__host__ inline void resetBufferCollabRW_BM() { pbm_pp_reset(PBM_PP_CORW_BM); }

/* ---- Random Walk + bitmap (parallelPage.cu:1042-1182) ---- */
__host__ inline void initPagesRandomWalk_BM() { pbm_pp_init(PBM_PP_RW_BM, false); }
__device__ inline int getPageRandomWalk_BM(int* step_count = 0) {
    const auto& d = pbm_pp_dev[PBM_PP_RW_BM];
    return d.valid ? pbm::walk_word<uint32_t>(d.view, pbm::dropin::call_seed(), PBM_DROPIN_MAX_STEPS, step_count)
                   : -1;
}
__device__ inline int getXPageRandomWalk_BM(int X, int* step_count = 0) {
    const auto& d = pbm_pp_dev[PBM_PP_RW_BM];
    if (!d.valid || X < 1 || X > 32) return -1;
    return pbm::walk_run(d.view, (uint32_t)X, pbm::dropin::call_seed(), PBM_DROPIN_MAX_STEPS, step_count);
}
__device__ inline void freePageRandomWalk_BM(int pageID) {
    pbm::dropin::free_checked(pbm_pp_dev[PBM_PP_RW_BM], pageID);
}
__host__ inline void printNumPagesLeftRandomWalk_BM() { pbm_pp_print(PBM_PP_RW_BM, "RW"); }
__host__ inline void resetBufferRandomWalk_BM() { pbm_pp_reset(PBM_PP_RW_BM); }

/* ---- Clustered Random Walk + bitmap (parallelPage.cu:1185-1320) ---- */
__host__ inline void initPagesClusteredRandomWalk_BM() { pbm_pp_init(PBM_PP_CRW_BM, false); }
__device__ inline int getPageClusteredRandomWalk_BM(int* step_count = 0) {
    const auto& d = pbm_pp_dev[PBM_PP_CRW_BM];
    if (!d.valid) return -1;
    int32_t* cur = d.cursors + ((uint32_t)pbm_pp_tid() % d.max_slots);
    int32_t c = *cur;
    int id = pbm::walk_crw(d.view, &c, pbm::dropin::call_seed(), PBM_DROPIN_MAX_STEPS, step_count);
    *cur = c;
    return id;
}
/* declared but never defined by the reference (parallelPage.cuh:72) */
__device__ inline int getXPageClusteredRandomWalk_BM(int X, int* step_count = 0) {
    const auto& d = pbm_pp_dev[PBM_PP_CRW_BM];
    if (!d.valid || X < 1 || X > 32) return -1;
    return pbm::walk_run(d.view, (uint32_t)X, pbm::dropin::call_seed(), PBM_DROPIN_MAX_STEPS, step_count);
}
__device__ inline void freePageClusteredRandomWalk_BM(int pageID) {
    pbm::dropin::free_checked(pbm_pp_dev[PBM_PP_CRW_BM], pageID);
}
__host__ inline void printNumPagesLeftClusteredRandomWalk_BM() { pbm_pp_print(PBM_PP_CRW_BM, "CRW_BM"); }
__host__ inline void resetBufferClusteredRandomWalk_BM() { pbm_pp_reset(PBM_PP_CRW_BM); }

/* gpuErrchk: parallelPage.cuh:79-86 (reports instead of exit()) */
#ifndef gpuErrchk
#define gpuErrchk(ans) pbm_gpu_report((ans), __FILE__, __LINE__)
inline void pbm_gpu_report(cudaError_t code, const char* file, int line) {
    if (code != cudaSuccess) std::fprintf(stderr, "GPUassert: %s %s %d\n", cudaGetErrorString(code), file, line);
}
#endif
