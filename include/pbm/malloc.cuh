// Drop-in for source/malloc.cuh (+ malloc.cu): MemoryManager,
// KernelMallocSimple and KernelMallocCollab with host constructors and
// device malloc(int) / free(void*), passed by value into a caller's kernels.
//
// All three share the size-classed allocator of pbm/pbm_malloc.cuh over a
// pool of PBM_MALLOC_POOL_PAGES pages of PBM_MALLOC_PAGE_SIZE bytes (power of
// two, 2 KiB .. 64 KiB; the reference's 264-byte pages cannot hold its own
// 64 KiB-class chunks).  Differences from the reference, by design: free()
// releases memory (KernelMallocSimple::free is empty in the reference,
// malloc.cu:157-159, and KernelMallocCollab frees only whole chunks,
// malloc.cu:300-320); the destructor leaves the pool alive because kernel
// arguments are copies of the object -- call release() to free it.
#pragma once
#include <climits>

#include "pbm/dropin.cuh"
#include "pbm/pbm_malloc.cuh"

#ifndef PBM_MALLOC_PAGE_SIZE
#define PBM_MALLOC_PAGE_SIZE 4096
#endif
#ifndef PBM_MALLOC_POOL_PAGES
#define PBM_MALLOC_POOL_PAGES (1u << 21)   // 8 GiB of 4 KiB pages
#endif

class MemoryManager {
public:
    /* MemoryManager(maxNThreads): malloc.cuh:6, malloc.cu:15-19 */
    __host__ MemoryManager(int _maxNThreads = INT_MAX) : m_maxNThreads(_maxNThreads) {
        pbm_pool_config c{};
        c.n_pages = PBM_MALLOC_POOL_PAGES;
        c.page_size = PBM_MALLOC_PAGE_SIZE;
        c.flags = PBM_POOL_MATERIALIZE;
        m_pool = nullptr;
        m_view = pbm::MallocView{};
        if (pbm_pool_create(&c, &m_pool) != PBM_OK || pbm_malloc_init(m_pool) != PBM_OK) {
            std::fprintf(stderr, "[pbm] MemoryManager: pool could not be created\n");
            if (m_pool) pbm_pool_destroy(m_pool);
            m_pool = nullptr;
            return;
        }
        pbm_device_state d{};
        pbm_pool_device_state(m_pool, 0, &d, nullptr);
        pbm_malloc_tables(m_pool, (void**)&m_view.start_of, (void**)&m_view.live, (void**)&m_view.len_of);
        m_view.pool.words = (uint32_t*)d.words;
        m_view.pool.base = (char*)d.base;
        m_view.pool.n_pages = (uint32_t)d.n_pages;
        m_view.pool.n_words32 = d.n_words32;
        m_view.pool.n_words64 = d.n_words64;
        m_view.pool.page_size = d.page_size;
        uint32_t sh = 0;
        while ((1u << sh) < d.page_size) ++sh;
        m_view.page_shift = sh;
    }
    __host__ ~MemoryManager() {}
    /* reset(): free all memory (malloc.cu:82-86, 214-216) */
    __host__ void reset() {
        if (!m_pool) return;
        pbm_malloc_release(m_pool);
        pbm_pool_reset(m_pool, nullptr);
        pbm_malloc_init(m_pool);
        pbm_malloc_tables(m_pool, (void**)&m_view.start_of, (void**)&m_view.live, (void**)&m_view.len_of);
        cudaDeviceSynchronize();
    }
    /* frees the pool (no reference counterpart: its destructors are TODO) */
    __host__ void release() {
        if (m_pool) pbm_pool_destroy(m_pool);
        m_pool = nullptr;
        m_view = pbm::MallocView{};
    }
    /* malloc(size): the calling lanes must be converged; nullptr on failure */
    __device__ void* malloc(int size) {
        if (!m_view.start_of || size <= 0) return nullptr;
        const uint32_t active = __activemask();
        const int32_t own = pbm::dropin::call_seed();
        const int32_t shared = (__shfl_sync(active, own, __ffs((int)active) - 1) ^ 0x2545F491) & 0x7fffffff;
        return pbm::malloc_group(m_view, active, (uint64_t)size, shared, own, PBM_DROPIN_MAX_STEPS, false,
                                 nullptr);
    }
    /* free(addr): the calling lanes must be converged */
    __device__ void free(void* addr) {
        if (!m_view.start_of) return;
        pbm::free_group(m_view, __activemask(), addr);
    }
    __host__ float freePagePercentage() const {
        if (!m_pool) return 0.f;
        uint64_t used = 0;
        pbm_pool_used(m_pool, &used, nullptr);
        return (float)(PBM_MALLOC_POOL_PAGES - used) / (float)PBM_MALLOC_POOL_PAGES;
    }
    int m_maxNThreads;
    pbm::MallocView m_view;
    pbm_pool* m_pool;
};

/* KernelMallocSimple(maxNThreads): malloc.cuh:14-24, malloc.cu:61-160 */
class KernelMallocSimple : public MemoryManager {
public:
    __host__ KernelMallocSimple(int _maxNThreads) : MemoryManager(_maxNThreads) {}
};

/* KernelMallocCollab(): malloc.cuh:27-37, malloc.cu:201-320 */
class KernelMallocCollab : public MemoryManager {
public:
    __host__ KernelMallocCollab() : MemoryManager() {}
};
