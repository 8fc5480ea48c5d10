// pbm_malloc.cuh -- size-classed device malloc / free over the page pool.
//
// Restates the idea of the reference's mallocRW / freeRW (source/RWMalloc.cuh:
// 299-334) and KernelMallocCollab (source/malloc.cu:223-320) -- a warp's
// small requests share one run of contiguous pages -- with the leaks closed:
//
//   * sizes are rounded up to power-of-two classes, 16 B .. 64 KiB;
//   * requests of at least a page get their own run of size/page_size pages
//     (walk_span: the run may cross bitmap words, which the reference's
//     one-word find0Range cannot, RWMalloc.cuh:159-200);
//   * the sub-page requests of a group of 32 requests are packed into one run,
//     largest class first, so every sub-page block is aligned to its own size
//     (blocks of a page or more start on a page boundary);
//   * each run keeps a live-block count at its first page; a free decrements
//     it and the free that reaches zero releases the run (the reference's
//     non-leader blocks are never released, RWMalloc.cuh:331, and a leader's
//     free releases the whole run under its members);
//   * every page of a run records the run's first page, so free(ptr) finds
//     the run in O(1) (the reference scans the 1 GB groups, Paging.cuh:40-52).
//
// Side tables: start_of[T] int32, live[T] int32, len_of[T] uint8.
#pragma once
#include "pbm/pbm_device.cuh"

namespace pbm {

constexpr int kMallocMinShift = 4;     // 16 B
constexpr int kMallocMaxShift = 16;    // 64 KiB

struct MallocView {
    PoolView pool;
    int32_t* start_of;   // first page of the run holding this page
    int32_t* live;       // live blocks of the run (valid at a run's first page)
    uint8_t* len_of;     // pages of the run (valid at a run's first page)
    uint32_t page_shift; // log2(page_size)
};

// Size class of a request: 0 = 16 B ... 12 = 64 KiB; -1 = no request (0 B)
// or too large.
__host__ __device__ __forceinline__ int malloc_class(uint64_t size) {
    if (size == 0 || size > (1ull << kMallocMaxShift)) return -1;
    int c = 0;
    while ((1ull << (kMallocMinShift + c)) < size) ++c;
    return c;
}

#ifdef __CUDACC__

__device__ __forceinline__ void malloc_mark_run(const MallocView& m, int32_t start, uint32_t n, int32_t blocks) {
    for (uint32_t k = 0; k < n; ++k) m.start_of[start + (int32_t)k] = start;
    m.len_of[start] = (uint8_t)n;
    m.live[start] = blocks;
}

// One group of up to 32 lanes (all lanes of `active` call converged).  Each
// lane with size > 0 gets a block pointer or nullptr.  seed_small: LCG seed of
// the group's shared small run; seed_own: this lane's own seed (large runs).
// serial_large != 0 claims the large runs one lane at a time, in lane order
// (the deterministic form used by single-warp replays).
__device__ __forceinline__ void* malloc_group(const MallocView& m, uint32_t active, uint64_t size,
                                              int32_t seed_small, int32_t seed_own, uint32_t max_steps,
                                              bool serial_large, int32_t* steps_out) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t lt = (1u << lane) - 1u;
    const uint32_t page = 1u << m.page_shift;
    const int cls = malloc_class(size);
    const uint32_t bytes = cls >= 0 ? (1u << (kMallocMinShift + cls)) : 0u;
    const bool small = cls >= 0 && bytes < page;
    const bool large = cls >= 0 && bytes >= page;
    int32_t steps = 0;
    // pack the small blocks, largest class first (keeps every block aligned)
    uint32_t offset = 0, total = 0;
    const int max_small = (int)m.page_shift - 1 - kMallocMinShift;   // class of page/2
    for (int c = max_small; c >= 0; --c) {
        uint32_t mask = __ballot_sync(active, small && cls == c);
        if (small && cls == c) offset = total + (uint32_t)__popc(mask & lt) * (1u << (kMallocMinShift + c));
        total += (uint32_t)__popc(mask) << (kMallocMinShift + c);
    }
    void* out = nullptr;
    const uint32_t small_mask = __ballot_sync(active, small);
    if (!serial_large && active == kFull32) {
        // the whole warp walks for the group's small run (its first small lane
        // asks for it) and the large runs together: one jump each, then 32
        // jumps at a time for each run still unserved; runs of more than 32
        // pages walk on their own
        const int leader = small_mask ? __ffs((int)small_mask) - 1 : -1;
        uint32_t need = 0u;
        int32_t seed = seed_own;
        if (large) {
            need = bytes >> m.page_shift;
        } else if ((int)lane == leader) {
            need = (total + page - 1u) >> m.page_shift;
            seed = seed_small;
        }
        int32_t s = 0;
        int32_t start = walk_span_warp(m.pool, need <= 32u ? need : 0u, seed, max_steps, &s);
        if (need > 32u) start = walk_span(m.pool, need, seed, max_steps, &s);
        if (need) steps = s;
        if (start >= 0) malloc_mark_run(m, start, need, large ? 1 : __popc(small_mask));
        const int32_t small_start = __shfl_sync(kFull32, start, leader >= 0 ? leader : 0);
        if (small && small_start >= 0)
            out = (void*)(m.pool.base + ((size_t)(uint32_t)small_start << m.page_shift) + offset);
        if (large && start >= 0) out = (void*)(m.pool.base + ((size_t)(uint32_t)start << m.page_shift));
        if (steps_out) *steps_out = steps;
        return out;
    }
    if (small_mask) {
        const int leader = __ffs((int)small_mask) - 1;
        int32_t start = -1;
        if ((int)lane == leader) {
            const uint32_t n = (total + page - 1u) >> m.page_shift;
            start = walk_span(m.pool, n, seed_small, max_steps, &steps);
            if (start >= 0) malloc_mark_run(m, start, n, __popc(small_mask));
        }
        start = __shfl_sync(active, start, leader);
        if (small && start >= 0)
            out = (void*)(m.pool.base + ((size_t)(uint32_t)start << m.page_shift) + offset);
    }
    if (serial_large) {
        uint32_t lm = __ballot_sync(active, large);
        while (lm) {
            const int l = __ffs((int)lm) - 1;
            lm &= lm - 1u;
            if ((int)lane == l) {
                const uint32_t n = bytes >> m.page_shift;
                int32_t s = 0;
                const int32_t start = walk_span(m.pool, n, seed_own, max_steps, &s);
                steps += s;
                if (start >= 0) {
                    malloc_mark_run(m, start, n, 1);
                    out = (void*)(m.pool.base + ((size_t)(uint32_t)start << m.page_shift));
                }
            }
            __syncwarp(active);
        }
    } else if (large) {
        const uint32_t n = bytes >> m.page_shift;
        int32_t s = 0;
        const int32_t start = walk_span(m.pool, n, seed_own, max_steps, &s);
        steps += s;
        if (start >= 0) {
            malloc_mark_run(m, start, n, 1);
            out = (void*)(m.pool.base + ((size_t)(uint32_t)start << m.page_shift));
        }
    }
    if (steps_out) *steps_out = steps;
    return out;
}

// Free of one block per calling lane (nullptr = nothing).  Lanes freeing
// blocks of the same run merge their decrements; the decrement that reaches
// zero releases the run.  Returns false for a pointer outside the pool or a
// run with no live block (double free), which is then left untouched.
__device__ __forceinline__ bool free_group(const MallocView& m, uint32_t active, const void* ptr) {
    const uint32_t lane = threadIdx.x & 31u;
    int32_t run = -1;
    bool ok = true;
    if (ptr) {
        const char* p = (const char*)ptr;
        const size_t span = (size_t)m.pool.n_pages << m.page_shift;
        if (p < m.pool.base || (size_t)(p - m.pool.base) >= span) {
            ok = false;
        } else {
            const int32_t pg = (int32_t)((size_t)(p - m.pool.base) >> m.page_shift);
            run = __ldcg(m.start_of + pg);
        }
    }
    const uint32_t peers = __match_any_sync(active, (uint32_t)run);
    if (run >= 0 && (__ffs((int)peers) - 1) == (int)lane) {
        const int32_t k = __popc(peers);
        const int32_t old = atomicSub(m.live + run, k);
        if (old == k) {
            free_span(m.pool, run, m.len_of[run]);
        } else if (old < k) {
            atomicAdd(m.live + run, k);   // double free: undo, report
            ok = false;
        }
    }
    return __shfl_sync(active, ok ? 1 : 0, lane) != 0;
}

#endif  // __CUDACC__
}  // namespace pbm
