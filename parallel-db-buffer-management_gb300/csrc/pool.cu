// pool.cu -- page pool lifecycle, prefill, occupancy, snapshots, invariant
// checks and the free-list build.
//
// Reference counterparts: initPages/pageAddress/getPageID (source/Paging.cuh:30-85),
// initMemoryManagement/resetMemoryManager/getFreePagePercentage/prefillBuffer
// (source/RandomWalkBasic_BM.cuh:42-164 and copies), popc_kernel + cub sum
// (RandomWalkBasic_BM.cuh:109-145).
#include <cstdlib>
#include <cstring>
#include <new>

#include <atomic>

#include <algorithm>

#include "internal.cuh"

namespace pbm {

std::atomic<unsigned long long> g_launches{0};

// SM count of the current device, cached per device ordinal (one atomic
// word each, so host threads launching at once never see a torn value).
int sm_count() {
    static std::atomic<int> cached[64];
    int dev = 0;
    cudaGetDevice(&dev);
    std::atomic<int>* slot = (dev >= 0 && dev < 64) ? &cached[dev] : nullptr;
    int c = slot ? slot->load(std::memory_order_relaxed) : 0;
    if (!c) {
        int n = 0;
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        c = n > 0 ? n : 1;
        if (slot) slot->store(c, std::memory_order_relaxed);
    }
    return c;
}

// Whether a kernel may write p: device or managed memory, or host memory that
// is pinned and mapped (cudaHostAlloc, cudaHostRegister).  Plain pageable host
// memory is refused, so a wrong buffer is an error status and never a kernel
// touching an unmapped address.
bool device_writable(const void* p) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) return true;
    return at.type == cudaMemoryTypeHost && at.devicePointer == p;
}

// Bernoulli(occ) bitmap: one thread per 32-bit word, one hash per page.
__global__ void k_prefill(uint32_t* words, uint32_t n_words, uint64_t n_pages,
                          uint64_t thresh53, uint64_t seed) {
    for (uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; w < n_words;
         w += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t val = 0;
        uint64_t p0 = (uint64_t)w * 32u;
#pragma unroll 8
        for (uint32_t b = 0; b < 32; ++b) {
            uint64_t p = p0 + b;
            bool held = p >= n_pages || (hash64(seed, p) >> 11) < thresh53;
            val |= (uint32_t)held << b;
        }
        words[w] = val;
    }
}

// Padding bits only (reset): clear every word, then set bits >= n_pages.
__global__ void k_reset_words(uint32_t* words, uint32_t n_words, uint64_t n_pages) {
    for (uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; w < n_words;
         w += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t p0 = (uint64_t)w * 32u;
        uint32_t val = 0;
        if (p0 + 32u > n_pages) {
            for (uint32_t b = 0; b < 32; ++b) if (p0 + b >= n_pages) val |= 1u << b;
        }
        words[w] = val;
    }
}

// Sets the padding bits (pages >= n_pages) of the last words again, e.g.
// after a caller wrote the bitmap: the walks rely on them never being free.
__global__ void k_set_padding(uint32_t* words, uint32_t n_words, uint64_t n_pages) {
    const uint32_t w = (uint32_t)(n_pages >> 5) + threadIdx.x;
    if (w >= n_words) return;
    const uint64_t p0 = (uint64_t)w * 32u;
    uint32_t pad = 0;
    for (uint32_t b = 0; b < 32; ++b) if (p0 + b >= n_pages) pad |= 1u << b;
    if (pad) words[w] |= pad;
}

__device__ __forceinline__ unsigned long long warp_sum64(unsigned long long v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_down_sync(0xffffffffu, v, d);
    return v;  // valid in lane 0
}

// Block-wide sum (blockDim.x a multiple of 32, <= 1024); result in thread 0.
__device__ __forceinline__ unsigned long long block_sum(unsigned long long v) {
    __shared__ unsigned long long red[32];
    v = warp_sum64(v);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) red[warp] = v;
    __syncthreads();
    unsigned long long t = 0;
    if (warp == 0) {
        t = lane < (int)(blockDim.x >> 5) ? red[lane] : 0ull;
        t = warp_sum64(t);
    }
    __syncthreads();
    return t;
}

// Fused popcount-reduce over the bitmap (one pass, 64-bit words).
__global__ void k_popcount(const unsigned long long* words, uint32_t n_words64,
                           unsigned long long* out) {
    unsigned long long c = 0;
    for (uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; w < n_words64;
         w += (uint64_t)gridDim.x * blockDim.x)
        c += (unsigned long long)__popcll(__ldcg(words + w));
    c = block_sum(c);
    if (threadIdx.x == 0 && c) atomicAdd(out, c);
}

// Invariant check of an id list: range, duplicates (scratch bitmap `seen`),
// and that every returned page is marked held.
__global__ void k_check_ids(const uint32_t* words, uint32_t* seen, uint64_t n_pages,
                            const int32_t* ids, uint32_t n, CheckCounters* out) {
    unsigned long long ok = 0, failed = 0, oor = 0, dup = 0, unmarked = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        int32_t id = ids[i];
        if (id == -1) { ++failed; continue; }
        if (id < 0 || (uint64_t)id >= n_pages) { ++oor; continue; }
        ++ok;
        uint32_t w = (uint32_t)id >> 5, bit = 1u << ((uint32_t)id & 31u);
        if (atomicOr(seen + w, bit) & bit) ++dup;
        if (!(__ldcg(words + w) & bit)) ++unmarked;
    }
    ok = block_sum(ok);
    failed = block_sum(failed);
    oor = block_sum(oor);
    dup = block_sum(dup);
    unmarked = block_sum(unmarked);
    if (threadIdx.x == 0) {
        if (ok) atomicAdd(&out->ok, ok);
        if (failed) atomicAdd(&out->failed, failed);
        if (oor) atomicAdd(&out->out_of_range, oor);
        if (dup) atomicAdd(&out->duplicates, dup);
        if (unmarked) atomicAdd(&out->not_marked, unmarked);
    }
}

// ---- free-list build: the FIFO ring holds the free pages in ascending order ----
// pass 1: free pages per block of 32-bit words
__global__ void k_fifo_count(const uint32_t* words, uint32_t n_words, uint32_t words_per_block,
                             unsigned long long* counts) {
    uint32_t w0 = blockIdx.x * words_per_block;
    unsigned long long c = 0;
    for (uint32_t w = w0 + threadIdx.x; w < n_words && w < w0 + words_per_block; w += blockDim.x)
        c += (unsigned long long)__popc(~__ldcg(words + w));
    c = block_sum(c);
    if (threadIdx.x == 0) counts[blockIdx.x] = c;
}
// pass 2: exclusive scan of the per-block counts (one block)
__global__ void k_fifo_scan(unsigned long long* counts, uint32_t n_blocks, FifoState* st,
                            int32_t* ring, uint64_t n_pages) {
    if (threadIdx.x == 0) {
        unsigned long long acc = 0;
        for (uint32_t b = 0; b < n_blocks; ++b) {
            unsigned long long c = counts[b];
            counts[b] = acc;
            acc += c;
        }
        st->head = 0;
        st->tail = acc;
        st->avail = acc;
    }
}
// pass 3: each block writes its free pages; the rest of the ring is empty (-1)
__global__ void k_fifo_fill(const uint32_t* words, uint32_t n_words, uint32_t words_per_block,
                            const unsigned long long* offs, int32_t* ring, uint64_t n_pages) {
    uint32_t w0 = blockIdx.x * words_per_block;
    __shared__ unsigned long long base;
    if (threadIdx.x == 0) base = offs[blockIdx.x];
    __syncthreads();
    // sequential within the block by warps of words, ordered by word index
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    __shared__ unsigned long long warp_base[32];
    for (uint32_t chunk = w0; chunk < w0 + words_per_block && chunk < n_words;
         chunk += (uint32_t)nwarps * 32u) {
        uint32_t w = chunk + (uint32_t)warp * 32u + (uint32_t)lane;
        uint32_t fr = (w < n_words && w < w0 + words_per_block) ? ~__ldcg(words + w) : 0u;
        int c = __popc(fr);
        int incl = c;
        for (int d = 1; d < 32; d <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= d) incl += y;
        }
        if (lane == 31) warp_base[warp] = (unsigned long long)incl;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned long long acc = base;
            for (int i = 0; i < nwarps; ++i) { unsigned long long t = warp_base[i]; warp_base[i] = acc; acc += t; }
            base = acc;
        }
        __syncthreads();
        unsigned long long pos = warp_base[warp] + (unsigned long long)(incl - c);
        while (fr) {
            int b = __ffs((int)fr) - 1;
            fr &= fr - 1u;
            ring[pos++] = (int32_t)(w * 32u + (uint32_t)b);
        }
        __syncthreads();
    }
}
__global__ void k_fifo_clear_tail(int32_t* ring, const FifoState* st, uint64_t n_pages) {
    unsigned long long start = st->tail;
    for (unsigned long long i = start + blockIdx.x * blockDim.x + threadIdx.x; i < n_pages;
         i += (unsigned long long)gridDim.x * blockDim.x)
        ring[i] = -1;
}

int fifo_build(pbm_pool* pool, cudaStream_t s) {
    if (!pool->d_ring) {
        if (cudaMalloc(&pool->d_ring, sizeof(int32_t) * pool->n_pages) != cudaSuccess) {
            cudaGetLastError();
            pool->d_ring = nullptr;
            return PBM_ERR_NOMEM;
        }
    }
    const uint32_t nw = pool->view.n_words32;
    const uint32_t wpb = 4096;
    const uint32_t nb = (nw + wpb - 1) / wpb;
    k_fifo_count<<<nb, 256, 0, s>>>(pool->d_words, nw, wpb, pool->d_scan);
    PBM_LAUNCH_CHECK();
    k_fifo_scan<<<1, 32, 0, s>>>(pool->d_scan, nb, pool->d_fifo, pool->d_ring, pool->n_pages);
    PBM_LAUNCH_CHECK();
    k_fifo_fill<<<nb, 256, 0, s>>>(pool->d_words, nw, wpb, pool->d_scan, pool->d_ring, pool->n_pages);
    PBM_LAUNCH_CHECK();
    k_fifo_clear_tail<<<sm_count() * 4, 256, 0, s>>>(pool->d_ring, pool->d_fifo, pool->n_pages);
    PBM_LAUNCH_CHECK();
    pool->fifo_valid = true;
    return PBM_OK;
}

// ---- fail-fast launch budget ----
// Pass 1: the free pages (clear bits; padding bits stay set) of each block's
// contiguous slice of `per` 64-bit words, into counts[block] and the totals.
__global__ void k_free_budget(const unsigned long long* words, uint32_t n_words64, uint32_t per,
                              unsigned long long* counts, LaunchBudget* b) {
    const uint64_t w0 = (uint64_t)blockIdx.x * per;
    const uint64_t w1 = min((uint64_t)n_words64, w0 + per);
    unsigned long long c = 0;
    for (uint64_t w = w0 + threadIdx.x; w < w1; w += blockDim.x)
        c += (unsigned long long)__popcll(~__ldcg(words + w));
    c = block_sum(c);
    if (threadIdx.x == 0) {
        counts[blockIdx.x] = c;
        if (c) atomicAdd(reinterpret_cast<unsigned long long*>(&b->free_at_start), c);
    }
}

// Pass 2: when the launch asks for at least half of the F free pages and the
// list holds them, every block writes its slice's free pages in ascending
// order at its offset (the counts of the blocks before it); list_mode says
// whether the list is valid for this launch.
__global__ void k_free_list(const unsigned long long* words, uint32_t n_words64, uint32_t per,
                            const unsigned long long* counts, LaunchBudget* b, unsigned long long n_requests,
                            int32_t* list, unsigned long long cap) {
    __shared__ unsigned long long warp_tot[32];
    __shared__ unsigned long long s_base;
    const long long F = b->free_at_start;
    const bool mode = F > 0 && 2ull * n_requests >= (unsigned long long)F && (unsigned long long)F <= cap;
    if (blockIdx.x == 0 && threadIdx.x == 0) b->list_mode = mode ? 1 : 0;
    if (!mode) return;
    unsigned long long off = 0;
    for (uint32_t k = threadIdx.x; k < blockIdx.x; k += blockDim.x) off += counts[k];
    off = block_sum(off);
    if (threadIdx.x == 0) s_base = off;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const uint64_t w0 = (uint64_t)blockIdx.x * per;
    const uint64_t w1 = min((uint64_t)n_words64, w0 + per);
    for (uint64_t base = w0; base < w1; base += blockDim.x) {
        const uint64_t w = base + threadIdx.x;
        unsigned long long fr = w < w1 ? ~__ldcg(words + w) : 0ull;
        const int c = __popcll(fr);
        int incl = c;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= d) incl += y;
        }
        if (lane == 31) warp_tot[warp] = (unsigned long long)incl;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned long long acc = 0;
            for (int i = 0; i < nwarps; ++i) { const unsigned long long t = warp_tot[i]; warp_tot[i] = acc; acc += t; }
            warp_tot[31] = acc;   // (nwarps <= 8 here, so slot 31 is free) the chunk's total
        }
        __syncthreads();
        unsigned long long pos = s_base + warp_tot[warp] + (unsigned long long)(incl - c);
        while (fr) {
            const int bit = __ffsll((long long)fr) - 1;
            fr &= fr - 1ull;
            list[pos++] = (int32_t)(w * 64u + (uint64_t)bit);
        }
        __syncthreads();
        if (threadIdx.x == 0) s_base += warp_tot[31];
        __syncthreads();
    }
}

int budget_prepare(pbm_pool* pool, uint64_t n_requests, cudaStream_t s) {
    PBM_CUDA_TRY(cudaMemsetAsync(pool->d_budget, 0, sizeof(LaunchBudget), s));
    const uint32_t nw64 = (uint32_t)(pool->bitmap_bytes / 8u);
    const uint32_t nb = pool->budget_blocks;
    const uint32_t per = (nw64 + nb - 1u) / nb;
    k_free_budget<<<nb, 256, 0, s>>>(reinterpret_cast<const unsigned long long*>(pool->d_words), nw64, per,
                                     pool->d_budget_blocks, pool->d_budget);
    PBM_LAUNCH_CHECK();
    k_free_list<<<nb, 256, 0, s>>>(reinterpret_cast<const unsigned long long*>(pool->d_words), nw64, per,
                                   pool->d_budget_blocks, pool->d_budget, (unsigned long long)n_requests,
                                   pool->d_free_list, (unsigned long long)pool->free_list_cap);
    PBM_LAUNCH_CHECK();
    return PBM_OK;
}

int popcount_used(pbm_pool* pool, uint64_t* used, cudaStream_t s) {
    PBM_CUDA_TRY(cudaMemsetAsync(&pool->d_check->used, 0, sizeof(unsigned long long), s));
    uint32_t nw64 = (uint32_t)(pool->bitmap_bytes / 8u);
    int blocks = sm_count() * 4;
    k_popcount<<<blocks, 256, 0, s>>>(reinterpret_cast<const unsigned long long*>(pool->d_words), nw64,
                                      &pool->d_check->used);
    PBM_LAUNCH_CHECK();
    unsigned long long h = 0;
    PBM_CUDA_TRY(cudaMemcpyAsync(&h, &pool->d_check->used, sizeof(h), cudaMemcpyDeviceToHost, s));
    PBM_CUDA_TRY(cudaStreamSynchronize(s));
    *used = (uint64_t)(h - pool->padding_bits);
    return PBM_OK;
}

}  // namespace pbm

using namespace pbm;

static void pool_free_all(pbm_pool* p) {
    if (!p) return;
    cudaFree(p->d_words);
    cudaFree(p->d_base);
    cudaFree(p->d_stats);
    cudaFree(p->d_cursors);
    cudaFree(p->d_arms);
    cudaFree(p->d_arm);
    cudaFree(p->d_ring);
    cudaFree(p->d_fifo);
    cudaFree(p->d_seen);
    cudaFree(p->d_check);
    cudaFree(p->d_budget);
    cudaFree(p->d_free_list);
    cudaFree(p->d_budget_blocks);
    cudaFree(p->d_scan);
    cudaFree(p->d_prefix);
    delete p;
}

__global__ void k_init_slots(int32_t* cursors, uint32_t* arms, uint32_t max_slots, uint32_t n_pages) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < max_slots; i += (uint64_t)gridDim.x * blockDim.x) {
        cursors[i] = -1;
        // distributed clock: arm0 = idx(lcg(seed(0, slot)), T) (parallelPage.cu:546-555 randomises arms)
        arms[i] = idx_hi(lcg(request_seed(0u, i)), n_pages);
    }
}

static int pool_reset_impl(pbm_pool* p, cudaStream_t s) {
    const uint32_t nw = (uint32_t)(p->bitmap_bytes / 4u);
    k_reset_words<<<sm_count() * 4, 256, 0, s>>>(p->d_words, nw, p->n_pages);
    PBM_LAUNCH_CHECK();
    k_init_slots<<<sm_count() * 4, 256, 0, s>>>(p->d_cursors, p->d_arms, p->max_slots, (uint32_t)p->n_pages);
    PBM_LAUNCH_CHECK();
    PBM_CUDA_TRY(cudaMemsetAsync(p->d_stats, 0, sizeof(DevStats), s));
    PBM_CUDA_TRY(cudaMemsetAsync(p->d_arm, 0, sizeof(unsigned long long), s));
    p->fifo_valid = false;
    return PBM_OK;
}

extern "C" {

const char* pbm_version(void) { return "pbm-gb300 0.1 (sm_103a)"; }
uint64_t pbm_kernel_launches(void) { return (uint64_t)g_launches.load(); }
int pbm_device_sm_count(int* h_sms) {
    if (!h_sms) return PBM_ERR_INVALID;
    *h_sms = sm_count();
    return PBM_OK;
}

int pbm_pool_create(const pbm_pool_config* cfg, pbm_pool** out) {
    if (!cfg || !out) return PBM_ERR_INVALID;
    *out = nullptr;
    if (cfg->n_pages == 0 || cfg->n_pages > 0x7fffffffull || cfg->page_size == 0) return PBM_ERR_INVALID;
    pbm_pool* p = new (std::nothrow) pbm_pool();
    if (!p) return PBM_ERR_NOMEM;
    std::memset((void*)p, 0, sizeof(*p));
    p->n_pages = cfg->n_pages;
    p->page_size = cfg->page_size;
    p->flags = cfg->flags;
    p->max_slots = cfg->max_slots ? cfg->max_slots : (1u << 22);
    cudaGetDevice(&p->device);
    const uint64_t nw64 = (cfg->n_pages + 63u) / 64u;
    p->bitmap_bytes = (size_t)nw64 * 8u;
    p->padding_bits = nw64 * 64u - cfg->n_pages;
    p->view.n_pages = (uint32_t)cfg->n_pages;
    p->view.n_words32 = (uint32_t)((cfg->n_pages + 31u) / 32u);
    p->view.n_words64 = (uint32_t)nw64;
    p->view.page_size = cfg->page_size;
    const uint32_t nb_scan = (uint32_t)((p->view.n_words32 + 4095u) / 4096u) + 1u;
    p->prefix_cap = 0;
    // the budget pass: one block per 256 64-bit words, at most 4 per SM; its
    // free list covers launches into a pool at least half full
    p->budget_blocks = (uint32_t)std::min<uint64_t>((uint64_t)sm_count() * 4u, std::max<uint64_t>(1u, (nw64 + 255u) / 256u));
    p->free_list_cap = std::max<uint64_t>(1024u, cfg->n_pages / 2u);
    bool ok = cudaMalloc(&p->d_words, p->bitmap_bytes) == cudaSuccess &&
              cudaMalloc(&p->d_stats, sizeof(DevStats)) == cudaSuccess &&
              cudaMalloc(&p->d_cursors, sizeof(int32_t) * p->max_slots) == cudaSuccess &&
              cudaMalloc(&p->d_arms, sizeof(uint32_t) * p->max_slots) == cudaSuccess &&
              cudaMalloc(&p->d_arm, sizeof(unsigned long long)) == cudaSuccess &&
              cudaMalloc(&p->d_fifo, sizeof(FifoState)) == cudaSuccess &&
              cudaMalloc(&p->d_seen, p->bitmap_bytes) == cudaSuccess &&
              cudaMalloc(&p->d_check, sizeof(CheckCounters)) == cudaSuccess &&
              cudaMalloc(&p->d_budget, sizeof(LaunchBudget)) == cudaSuccess &&
              cudaMalloc(&p->d_free_list, sizeof(int32_t) * p->free_list_cap) == cudaSuccess &&
              cudaMalloc(&p->d_budget_blocks, sizeof(unsigned long long) * p->budget_blocks) == cudaSuccess &&
              cudaMalloc(&p->d_scan, sizeof(unsigned long long) * nb_scan) == cudaSuccess;
    if (ok && (cfg->flags & PBM_POOL_MATERIALIZE)) {
        ok = cudaMalloc(&p->d_base, (size_t)cfg->n_pages * cfg->page_size) == cudaSuccess;
    }
    if (!ok) {
        cudaGetLastError();
        pool_free_all(p);
        return PBM_ERR_NOMEM;
    }
    p->view.words = p->d_words;
    p->view.base = p->d_base;
    int rc = pool_reset_impl(p, 0);
    if (rc == PBM_OK && cudaStreamSynchronize(0) != cudaSuccess) rc = PBM_ERR_CUDA;
    if (rc != PBM_OK) { pool_free_all(p); return rc; }
    *out = p;
    return PBM_OK;
}

int pbm_pool_destroy(pbm_pool* pool) {
    PBM_ON_POOL_DEVICE(pool);
    if (!pool) return PBM_ERR_INVALID;
    cudaDeviceSynchronize();
    pbm_malloc_release(pool);   // malloc side tables, if any
    pool_free_all(pool);
    return PBM_OK;
}

int pbm_pool_info(const pbm_pool* pool, uint64_t* n_pages, uint32_t* page_size, void** d_bitmap,
                  size_t* bitmap_bytes, void** d_base) {
    if (!pool) return PBM_ERR_INVALID;
    if (n_pages) *n_pages = pool->n_pages;
    if (page_size) *page_size = pool->page_size;
    if (d_bitmap) *d_bitmap = pool->d_words;
    if (bitmap_bytes) *bitmap_bytes = pool->bitmap_bytes;
    if (d_base) *d_base = pool->d_base;
    return PBM_OK;
}

int pbm_pool_reset(pbm_pool* pool, void* stream) {
    PBM_ON_POOL_DEVICE(pool);
    if (!pool) return PBM_ERR_INVALID;
    return pool_reset_impl(pool, (cudaStream_t)stream);
}

int pbm_pool_prefill_bernoulli(pbm_pool* pool, double occupancy, uint64_t seed, void* stream) {
    PBM_ON_POOL_DEVICE(pool);
    if (!pool || !(occupancy >= 0.0) || occupancy > 1.0) return PBM_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    uint64_t thresh = occupancy <= 0.0 ? 0ull
                      : occupancy >= 1.0 ? (1ull << 53)
                                         : (uint64_t)(occupancy * 9007199254740992.0);
    const uint32_t nw = (uint32_t)(pool->bitmap_bytes / 4u);
    k_prefill<<<sm_count() * 8, 256, 0, s>>>(pool->d_words, nw, pool->n_pages, thresh, seed);
    PBM_LAUNCH_CHECK();
    pool->fifo_valid = false;
    return PBM_OK;
}

int pbm_pool_used(pbm_pool* pool, uint64_t* h_used, void* stream) {
    PBM_ON_POOL_DEVICE(pool);
    if (!pool || !h_used) return PBM_ERR_INVALID;
    return popcount_used(pool, h_used, (cudaStream_t)stream);
}

int pbm_pool_read_bitmap(pbm_pool* pool, void* h_dst, size_t bytes, void* stream) {
    PBM_ON_POOL_DEVICE(pool);
    if (!pool || !h_dst || bytes != pool->bitmap_bytes) return PBM_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    PBM_CUDA_TRY(cudaMemcpyAsync(h_dst, pool->d_words, bytes, cudaMemcpyDeviceToHost, s));
    PBM_CUDA_TRY(cudaStreamSynchronize(s));
    return PBM_OK;
}

int pbm_pool_write_bitmap(pbm_pool* pool, const void* h_src, size_t bytes, void* stream) {
    PBM_ON_POOL_DEVICE(pool);
    if (!pool || !h_src || bytes != pool->bitmap_bytes) return PBM_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    PBM_CUDA_TRY(cudaMemcpyAsync(pool->d_words, h_src, bytes, cudaMemcpyHostToDevice, s));
    k_set_padding<<<1, 64, 0, s>>>(pool->d_words, (uint32_t)(bytes / 4u), pool->n_pages);
    PBM_LAUNCH_CHECK();
    PBM_CUDA_TRY(cudaStreamSynchronize(s));
    pool->fifo_valid = false;
    return PBM_OK;
}

int pbm_pool_device_state(pbm_pool* pool, int build_fifo, pbm_device_state* h_out, void* stream) {
    PBM_ON_POOL_DEVICE(pool);
    if (!pool || !h_out) return PBM_ERR_INVALID;
    if (build_fifo && !pool->fifo_valid) {
        int rc = fifo_build(pool, (cudaStream_t)stream);
        if (rc) return rc;
        PBM_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    }
    h_out->words = pool->d_words;
    h_out->base = pool->d_base;
    h_out->n_pages = pool->n_pages;
    h_out->page_size = pool->page_size;
    h_out->n_words32 = pool->view.n_words32;
    h_out->n_words64 = pool->view.n_words64;
    h_out->max_slots = pool->max_slots;
    h_out->cursors = pool->d_cursors;
    h_out->arms = pool->d_arms;
    h_out->single_arm = pool->d_arm;
    h_out->fifo_state = pool->d_fifo;
    h_out->fifo_ring = pool->d_ring;
    h_out->stats = pool->d_stats;
    return PBM_OK;
}

int pbm_pool_stats(pbm_pool* pool, pbm_stats* h_out, void* stream) {
    PBM_ON_POOL_DEVICE(pool);
    if (!pool || !h_out) return PBM_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    DevStats d;
    PBM_CUDA_TRY(cudaMemcpyAsync(&d, pool->d_stats, sizeof(d), cudaMemcpyDeviceToHost, s));
    PBM_CUDA_TRY(cudaStreamSynchronize(s));
    h_out->successes = d.successes;
    h_out->failures = d.failures;
    h_out->steps = d.steps;
    h_out->frees = d.frees;
    return d.timeouts ? PBM_ERR_TIMEOUT : PBM_OK;
}

int pbm_check_ids(pbm_pool* pool, const int32_t* d_ids, uint32_t n, pbm_check_result* h_out,
                  void* stream) {
    PBM_ON_POOL_DEVICE(pool);
    if (!pool || !h_out || (n && !d_ids)) return PBM_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    PBM_CUDA_TRY(cudaMemsetAsync(pool->d_seen, 0, pool->bitmap_bytes, s));
    PBM_CUDA_TRY(cudaMemsetAsync(pool->d_check, 0, sizeof(CheckCounters), s));
    if (n) {
        int blocks = (int)((n + 255u) / 256u);
        if (blocks > sm_count() * 8) blocks = sm_count() * 8;
        k_check_ids<<<blocks, 256, 0, s>>>(pool->d_words, pool->d_seen, pool->n_pages, d_ids, n,
                                           pool->d_check);
        PBM_LAUNCH_CHECK();
    }
    CheckCounters c;
    PBM_CUDA_TRY(cudaMemcpyAsync(&c, pool->d_check, sizeof(c), cudaMemcpyDeviceToHost, s));
    PBM_CUDA_TRY(cudaStreamSynchronize(s));
    uint64_t used = 0;
    int rc = popcount_used(pool, &used, s);
    if (rc) return rc;
    h_out->n_ok = (int64_t)c.ok;
    h_out->n_failed = (int64_t)c.failed;
    h_out->n_out_of_range = (int64_t)c.out_of_range;
    h_out->n_duplicates = (int64_t)c.duplicates;
    h_out->n_not_marked = (int64_t)c.not_marked;
    h_out->used_pages = (int64_t)used;
    return (c.out_of_range || c.duplicates || c.not_marked) ? PBM_ERR_CORRUPT : PBM_OK;
}

}  // extern "C"
