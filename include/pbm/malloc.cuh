// Drop-in for source/malloc.cuh (+ malloc.cu): MemoryManager,
// KernelMallocSimple and KernelMallocCollab with host constructors and
// device malloc(int) / free(void*), passed by value into a caller's kernels.
//
// All three allocate from one pool of PBM_MALLOC_POOL_PAGES pages of
// PBM_MALLOC_PAGE_SIZE bytes (power of two, 2 KiB .. 64 KiB; the reference's
// 264-byte pages cannot hold its own 64 KiB-class chunks), each run of pages
// carrying a live-block count:
//   * MemoryManager and KernelMallocCollab: the lanes of a warp pack their
//     sub-page requests into one shared run, larger requests get runs of
//     their own (pbm/pbm_malloc.cuh; the reference's warp suffix sum,
//     malloc.cu:223-289);
//   * KernelMallocSimple: each thread bumps through a chunk of its own and
//     claims a new one when the next request does not fit (malloc.cu:100-152).
// Differences from the reference, by design: free() releases memory
// (KernelMallocSimple::free is empty in the reference, malloc.cu:157-159,
// and KernelMallocCollab frees only whole chunks, malloc.cu:300-320); the
// destructor leaves the pool alive because kernel arguments are copies of the
// object -- call release() to free it.
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

/* KernelMallocSimple(maxNThreads): malloc.cuh:14-24, malloc.cu:61-160.
 * Each thread (global id below maxNThreads) keeps a chunk -- a run of pages
 * -- and bumps through it: a malloc that fits the rest of the chunk takes its
 * next bytes (16-byte aligned); one that does not retires the chunk and
 * claims a new run just large enough for the request (malloc.cu:100-152),
 * whose leftover serves the thread's next small requests.  Every block counts
 * as live in its run and the thread's hold on its current chunk counts once
 * more, so a run goes back to the pool when its last block is freed and its
 * thread has moved on to another chunk or called retire(). */
class KernelMallocSimple : public MemoryManager {
public:
    __host__ KernelMallocSimple(int _maxNThreads) : MemoryManager(_maxNThreads) {
        m_threads = _maxNThreads > 0 ? _maxNThreads : 0;
        m_chunk = nullptr;
        if (m_pool && m_threads) {
            if (cudaMalloc(&m_chunk, sizeof(int2) * (size_t)m_threads) != cudaSuccess) {
                cudaGetLastError();
                m_chunk = nullptr;
            } else {
                clear_chunks();
            }
        }
    }
    /* reset(): free all memory (malloc.cu:82-86) */
    __host__ void reset() {
        MemoryManager::reset();
        clear_chunks();
    }
    __host__ void release() {
        cudaFree(m_chunk);
        m_chunk = nullptr;
        MemoryManager::release();
    }
    /* malloc(size): nullptr on failure, for a thread at or past maxNThreads,
     * or for a request above 255 pages */
    __device__ void* malloc(int size) {
        if (!m_view.start_of || !m_chunk || size <= 0) return nullptr;
        const uint32_t tid = pbm::dropin::global_tid();
        if (tid >= (uint32_t)m_threads) return nullptr;
        const int2 st = m_chunk[tid];   // x: first page of the chunk (-1 none), y: bytes handed out
        const uint32_t bytes = ((uint32_t)size + 15u) & ~15u;
        const uint32_t page = m_view.pool.page_size;
        if (st.x >= 0) {
            const uint32_t cap = (uint32_t)m_view.len_of[st.x] * page;
            if ((uint32_t)st.y + bytes <= cap) {
                atomicAdd(m_view.live + st.x, 1);
                m_chunk[tid] = make_int2(st.x, st.y + (int)bytes);
                return m_view.pool.base + ((size_t)(uint32_t)st.x << m_view.page_shift) + st.y;
            }
            drop_chunk(st.x);
        }
        m_chunk[tid] = make_int2(-1, 0);
        const uint32_t n = (bytes + page - 1u) / page;
        if (n > 255u) return nullptr;
        int32_t steps = 0;
        const int32_t start = pbm::walk_span(m_view.pool, n, pbm::dropin::call_seed(), PBM_DROPIN_MAX_STEPS, &steps);
        if (start < 0) return nullptr;
        pbm::malloc_mark_run(m_view, start, n, 2);   // the block, and the thread's hold on its chunk
        m_chunk[tid] = make_int2(start, (int)bytes);
        return m_view.pool.base + ((size_t)(uint32_t)start << m_view.page_shift);
    }
    /* free(addr): the block's run loses one live block; the calling lanes
     * must be converged */
    __device__ void free(void* addr) { MemoryManager::free(addr); }
    /* retire(): the calling thread lets go of its current chunk, which goes
     * back to the pool once its blocks are freed (no reference counterpart) */
    __device__ void retire() {
        if (!m_chunk) return;
        const uint32_t tid = pbm::dropin::global_tid();
        if (tid >= (uint32_t)m_threads) return;
        const int2 st = m_chunk[tid];
        if (st.x >= 0) drop_chunk(st.x);
        m_chunk[tid] = make_int2(-1, 0);
    }
    int m_threads;
    int2* m_chunk;   // per thread: first page of its chunk and the bytes handed out

private:
    __device__ void drop_chunk(int32_t start) {
        if (atomicSub(m_view.live + start, 1) == 1) pbm::free_span(m_view.pool, start, m_view.len_of[start]);
    }
    __host__ void clear_chunks() {
        if (m_chunk) cudaMemset(m_chunk, 0xff, sizeof(int2) * (size_t)m_threads);   // no chunk
        cudaDeviceSynchronize();
    }
};

/* KernelMallocCollab(): malloc.cuh:27-37, malloc.cu:201-320.  The lanes of
 * a warp pack their sub-page requests into one shared run (largest class
 * first, so each block is aligned to its class); requests of a page or more
 * get runs of their own.  A run goes back to the pool with its last block. */
class KernelMallocCollab : public MemoryManager {
public:
    __host__ KernelMallocCollab() : MemoryManager() {}
};
