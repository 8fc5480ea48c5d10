// pbm_qmalloc.cuh -- queue-based size-class allocator over the page pool.
//
// An alternative backend for the size classes of pbm_malloc.cuh, in the
// manner of the page queues of the allocator the reference vendors as its
// comparator (Ouroboros, source/Ouroboros/include/device/queues/page/
// PageQueueVL_impl.cuh): every class (16 B .. 64 KiB, powers of two) keeps a
// FIFO ring of its free blocks.
//
//   malloc: the lanes of a warp asking for one class take their blocks from
//           its ring with one reservation and one ticket; lanes the ring
//           cannot serve carve fresh chunks from the page pool (spanning
//           walk), take blocks from them and enqueue the rest;
//   free:   the block goes back to its class's ring (the class of every
//           page of a chunk is recorded when the chunk is carved).
//
// A chunk is one page for classes below a page and one block for larger
// classes.  Chunks stay with their class: the rings are the free lists, and
// pages return to the pool only when the allocator is reset.  A block is
// named by a 32-bit handle, its byte offset in the pool / 16, so pools up to
// 64 GiB.  Rings are bounded MPMC queues with ticket counters: `avail` counts
// published blocks, `space` free slots; every wait on a slot is bounded and
// records a timeout.  A free into a full ring drops the block (counted).
// Frees are not checked for doubles (neither are the vendored allocator's).
#pragma once
#include "pbm/pbm_malloc.cuh"

namespace pbm {

constexpr int kQClasses = kMallocMaxShift - kMallocMinShift + 1;   // 13
constexpr uint32_t kEmptyHandle = 0xffffffffu;
constexpr uint32_t kQSpinLimit = 1u << 16;
constexpr uint8_t kQCont = 0x80u;   // class_of mark of a chunk's pages after its first

// Each counter sits in a 128-byte line of its own: every warp that mallocs
// or frees a class touches its counters, and counters that shared a line
// (or classes that shared one) queued their atomics at one L2 slice.
struct QueueRing {
    alignas(128) unsigned long long head;    // next dequeue ticket
    alignas(128) unsigned long long tail;    // next enqueue ticket
    alignas(128) unsigned long long avail;   // blocks published (signed, two's complement)
    alignas(128) unsigned long long space;   // free slots (signed, two's complement)
};

// counters[] indices, one 128-byte line apart (kQCounterWords words in all)
constexpr int kQChunks = 0, kQOverflow = 16, kQTimeouts = 32, kQBadFrees = 48;
constexpr int kQCounterWords = 64;

struct QMallocView {
    PoolView pool;
    QueueRing* rings;            // kQClasses
    uint32_t* slots;             // kQClasses * capacity handles
    uint8_t* class_of;           // per page: class + 1 of its chunk, | kQCont past the chunk's first page
                                 // (0 = no chunk)
    unsigned long long* counters;
    uint32_t capacity;           // slots per ring (power of two)
    uint32_t page_shift;
};

#ifdef __CUDACC__

__device__ __forceinline__ uint32_t q_chunk_bytes(const QMallocView& q, int cls) {
    const uint32_t b = 1u << (kMallocMinShift + cls);
    const uint32_t page = 1u << q.page_shift;
    return b > page ? b : page;
}

// Reserve up to k from a signed counter; returns how many were reserved.
__device__ __forceinline__ uint32_t q_reserve(unsigned long long* ctr, uint32_t k) {
    const long long old = (long long)atomicAdd(ctr, 0ull - (unsigned long long)k);
    const long long got = old <= 0 ? 0 : (old < (long long)k ? old : (long long)k);
    if ((long long)k > got) atomicAdd(ctr, (unsigned long long)((long long)k - got));
    return (uint32_t)got;
}

// Writes `h` into the ring slot of ticket t (bounded wait for the slot to
// be vacated by the dequeue of the previous lap).
__device__ __forceinline__ bool q_put_slot(const QMallocView& q, int cls, unsigned long long t, uint32_t h) {
    uint32_t* slot = q.slots + (size_t)cls * q.capacity + (uint32_t)(t & (q.capacity - 1u));
    for (uint32_t k = 0; k < kQSpinLimit; ++k) {
        if (atomicCAS(slot, kEmptyHandle, h) == kEmptyHandle) return true;
        __nanosleep(32);
    }
    atomicAdd(q.counters + kQTimeouts, 1ull);
    return false;
}

__device__ __forceinline__ uint32_t q_take_slot(const QMallocView& q, int cls, unsigned long long t) {
    uint32_t* slot = q.slots + (size_t)cls * q.capacity + (uint32_t)(t & (q.capacity - 1u));
    for (uint32_t k = 0; k < kQSpinLimit; ++k) {
        const uint32_t h = atomicExch(slot, kEmptyHandle);
        if (h != kEmptyHandle) return h;
        __nanosleep(32);
    }
    atomicAdd(q.counters + kQTimeouts, 1ull);
    return kEmptyHandle;
}

// One lane enqueues handles first, first+stride, ... (n of them) of one
// class; returns how many went in (the rest overflowed).
__device__ __forceinline__ uint32_t q_enqueue_run(const QMallocView& q, int cls, uint32_t first, uint32_t stride,
                                                  uint32_t n) {
    if (n == 0) return 0;
    QueueRing* r = q.rings + cls;
    const uint32_t got = q_reserve(&r->space, n);
    if (got < n) atomicAdd(q.counters + kQOverflow, (unsigned long long)(n - got));
    if (got == 0) return 0;
    const unsigned long long t0 = atomicAdd(&r->tail, (unsigned long long)got);
    uint32_t put = 0;
    for (uint32_t i = 0; i < got; ++i) put += q_put_slot(q, cls, t0 + i, first + i * stride) ? 1u : 0u;
    __threadfence();
    atomicAdd(&r->avail, (unsigned long long)put);
    return put;
}

__device__ __forceinline__ void* q_handle_ptr(const QMallocView& q, uint32_t h) {
    return (void*)(q.pool.base + (size_t)h * 16u);
}

// Marks a claimed chunk (first page `chunk`) as class `cls`, for refill lane
// `ri` of `r_total` (b blocks per chunk), and enqueues the blocks no refill
// lane takes.
__device__ __forceinline__ void q_carve_finish(const QMallocView& q, int cls, uint32_t ri, uint32_t r_total,
                                               uint32_t b, int32_t chunk) {
    const uint32_t npages = q_chunk_bytes(q, cls) >> q.page_shift;
    q.class_of[(uint32_t)chunk] = (uint8_t)(cls + 1);
    for (uint32_t p = 1; p < npages; ++p) q.class_of[(uint32_t)chunk + p] = (uint8_t)(kQCont | (cls + 1));
    atomicAdd(q.counters + kQChunks, 1ull);
    const uint32_t bytes = 1u << (kMallocMinShift + cls);
    const uint32_t first = (uint32_t)(((size_t)(uint32_t)chunk << q.page_shift) >> 4);
    const uint32_t users = r_total - ri < b ? r_total - ri : b;   // refill lanes served by this chunk
    q_enqueue_run(q, cls, first + users * (bytes >> 4), bytes >> 4, b - users);
}

// Carves one chunk of class `cls` (walk, then q_carve_finish); returns the
// chunk's first page or -1.
__device__ __forceinline__ int32_t q_carve(const QMallocView& q, int cls, uint32_t ri, uint32_t r_total, uint32_t b,
                                           int32_t seed_own, uint32_t max_steps, int32_t* steps) {
    const uint32_t npages = q_chunk_bytes(q, cls) >> q.page_shift;
    const int32_t chunk = walk_span(q.pool, npages, seed_own, max_steps, steps);
    if (chunk < 0) return -1;
    q_carve_finish(q, cls, ri, r_total, b, chunk);
    return chunk;
}

// malloc of one block per calling lane (size 0 = none); all lanes of
// `active` call converged.  seed_own: the lane's walk seed for a chunk it
// carves.  Returns the block or nullptr.  serial != 0 carves one lane at a
// time in lane order (the deterministic form used by one-warp replays).
__device__ __forceinline__ void* qmalloc_group(const QMallocView& q, uint32_t active, uint64_t size,
                                               int32_t seed_own, uint32_t max_steps, bool serial,
                                               int32_t* steps_out) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t lt = (1u << lane) - 1u;
    const int cls = malloc_class(size);
    const uint32_t key = cls >= 0 ? (uint32_t)cls : 0x100u + lane;   // lanes without a request never group
    const uint32_t peers = __match_any_sync(active, key);
    const uint32_t leader = (uint32_t)__ffs((int)peers) - 1u;
    const uint32_t k = (uint32_t)__popc(peers);
    const uint32_t rank = (uint32_t)__popc(peers & lt);
    int32_t steps = 0;
    void* out = nullptr;
    // 1. blocks from the class ring
    uint32_t got = 0;
    unsigned long long h0 = 0;
    if (cls >= 0 && lane == leader) {
        got = q_reserve(&q.rings[cls].avail, k);
        if (got) h0 = atomicAdd(&q.rings[cls].head, (unsigned long long)got);
    }
    got = __shfl_sync(active, got, (int)leader);
    h0 = __shfl_sync(active, h0, (int)leader);
    if (cls >= 0 && rank < got) {
        const uint32_t h = q_take_slot(q, cls, h0 + rank);
        if (h != kEmptyHandle) out = q_handle_ptr(q, h);
    }
    __syncwarp(active);
    if (cls >= 0 && lane == leader && got) {
        __threadfence();
        atomicAdd(&q.rings[cls].space, (unsigned long long)got);
    }
    // 2. the rest carve chunks: refill lane i of a class takes block i % b of
    //    the class's chunk i / b, carved by refill lane (i / b) * b, which
    //    also enqueues the blocks of its chunk that no lane takes
    const bool refill = cls >= 0 && rank >= got;
    const uint32_t b = cls >= 0 ? q_chunk_bytes(q, cls) >> (kMallocMinShift + cls) : 1u;
    const uint32_t ri = rank - got;                                   // refill index
    const uint32_t r_total = k - got;
    const bool carver = refill && ri % b == 0u;
    int32_t chunk = -1;                                               // first page of the carved chunk
    if (serial) {
        uint32_t cm = __ballot_sync(active, carver);
        while (cm) {
            const uint32_t l = (uint32_t)__ffs((int)cm) - 1u;
            cm &= cm - 1u;
            if (lane == l) chunk = q_carve(q, cls, ri, r_total, b, seed_own, max_steps, &steps);
            __syncwarp(active);
        }
    } else if (active == kFull32) {
        // the warp walks for all its chunks together (walk_span_warp); chunks
        // of more than 32 pages walk on their own
        const uint32_t npages = carver ? q_chunk_bytes(q, cls) >> q.page_shift : 0u;
        chunk = walk_span_warp(q.pool, npages <= 32u ? npages : 0u, seed_own, max_steps, &steps);
        if (npages > 32u) chunk = walk_span(q.pool, npages, seed_own, max_steps, &steps);
        if (!carver) steps = 0;
        if (chunk >= 0) q_carve_finish(q, cls, ri, r_total, b, chunk);
    } else if (carver) {
        chunk = q_carve(q, cls, ri, r_total, b, seed_own, max_steps, &steps);
    }
    // the carver of refill lane i is the refill lane (i / b) * b of the same class
    const uint32_t refill_mask = __ballot_sync(active, refill) & peers;
    uint32_t src = lane;
    if (refill) src = nth_set_bit(refill_mask, (int)((ri / b) * b));
    const int32_t base = __shfl_sync(active, chunk, (int)(refill ? src : lane));
    if (refill && base >= 0) {
        const uint32_t bytes = 1u << (kMallocMinShift + cls);
        out = (void*)(q.pool.base + ((size_t)(uint32_t)base << q.page_shift) + (size_t)(ri % b) * bytes);
    }
    if (steps_out) *steps_out = steps;
    return out;
}

// free of one block per calling lane (nullptr = nothing).  Returns false for
// a pointer outside the pool, not at a block start of its class, or on a
// page no chunk holds (those are left alone and counted).
__device__ __forceinline__ bool qfree_group(const QMallocView& q, uint32_t active, const void* ptr) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t lt = (1u << lane) - 1u;
    int cls = -1;
    uint32_t h = kEmptyHandle;
    bool ok = true;
    if (ptr) {
        const char* p = (const char*)ptr;
        const size_t span = (size_t)q.pool.n_pages << q.page_shift;
        const size_t off = (size_t)(p - q.pool.base);
        if (p < q.pool.base || off >= span || (off & 15u)) {
            ok = false;
        } else {
            const uint8_t mark = q.class_of[off >> q.page_shift];
            const int c1 = (int)(mark & (uint8_t)~kQCont) - 1;
            const uint32_t bytes = c1 >= 0 ? 1u << (kMallocMinShift + c1) : 0u;
            const uint32_t page = 1u << q.page_shift;
            const size_t align = bytes < page ? bytes : page;
            if (c1 < 0 || (mark & kQCont) || (off & (align - 1u))) ok = false;
            else { cls = c1; h = (uint32_t)(off >> 4); }
        }
        if (!ok) atomicAdd(q.counters + kQBadFrees, 1ull);
    }
    const uint32_t key = cls >= 0 ? (uint32_t)cls : 0x100u + lane;
    const uint32_t peers = __match_any_sync(active, key);
    const uint32_t leader = (uint32_t)__ffs((int)peers) - 1u;
    const uint32_t k = (uint32_t)__popc(peers);
    const uint32_t rank = (uint32_t)__popc(peers & lt);
    uint32_t got = 0;
    unsigned long long t0 = 0;
    if (cls >= 0 && lane == leader) {
        QueueRing* r = q.rings + cls;
        got = q_reserve(&r->space, k);
        if (got < k) atomicAdd(q.counters + kQOverflow, (unsigned long long)(k - got));
        if (got) t0 = atomicAdd(&r->tail, (unsigned long long)got);
    }
    got = __shfl_sync(active, got, (int)leader);
    t0 = __shfl_sync(active, t0, (int)leader);
    bool put = false;
    if (cls >= 0 && rank < got) {
        put = q_put_slot(q, cls, t0 + rank, h);
        __threadfence();
    }
    const uint32_t nput = (uint32_t)__popc(__ballot_sync(active, put) & peers);
    if (cls >= 0 && lane == leader && nput) {
        __threadfence();
        atomicAdd(&q.rings[cls].avail, (unsigned long long)nput);
    }
    return ok;
}

#endif  // __CUDACC__
}  // namespace pbm
