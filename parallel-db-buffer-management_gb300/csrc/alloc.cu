// alloc.cu -- page allocation and free kernels for every strategy.
//
// One launch serves n requests; request r uses LCG seed request_seed(seed, r)
// regardless of which thread runs it, so a one-thread (one-warp) launch of
// the same kernel is a deterministic replay of the same requests in order.
//
// Reference routines restated: getPage/freePage of RandomWalkBasic.cuh:54-84,
// RandomWalkBasic_BM.cuh:60-102, CollabRW_BM.cuh:114-160, CRW_BM.cuh:75-156;
// parallelPage.cu getPageLinkedList (:342-369), getPageSingleClock (:491-509),
// getPageDistClock (:571-592), getXPageRandomWalk_BM (:1104-1142).
#include "internal.cuh"

namespace pbm {

struct AllocArgs {
    PoolView v;
    uint32_t n;
    uint32_t seed;
    uint32_t max_steps;
    uint32_t stride;
    int32_t* ids;
    int32_t* steps;
    DevStats* stats;
    int32_t* cursors;            // clustered walk
    uint32_t* arms;              // distributed clock
    unsigned long long* arm;     // single clock
    uint32_t max_slots;
    int32_t dedupe;              // collaborative walk: W*stride may exceed L
    LaunchBudget* budget;        // fail-fast launch budget (null: every request walks)
    const int32_t* free_list;    // the budget's list of free pages (list mode)
};

// Per-thread accumulators reduced once per block.
struct Acc {
    unsigned long long ok = 0, fail = 0, steps = 0;
};

__device__ __forceinline__ void flush_acc(const Acc& a, DevStats* st) {
    block_add_counters<3>({a.ok, a.fail, a.steps}, {&st->successes, &st->failures, &st->steps});
}

enum class Walk { Page, Word32, Word64, Crw, SingleClock, DistClock };

// Per-thread strategies.  The loop runs whole warps (uniform trip count) so
// the block-level flush can use full-warp shuffles.
template <Walk K>
__global__ void __launch_bounds__(256) k_alloc_thread(AllocArgs a) {
    Acc acc;
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t nthr = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t n_round = ((uint64_t)a.n + 31u) & ~31ull;
    // whole warps iterate together (n_round and nthr are multiples of 32), or
    // one thread in the serial replay
    const bool listed = a.budget && __ldcg(&a.budget->list_mode);
    for (uint64_t r = tid; r < n_round; r += nthr) {
        const bool go = r < a.n && budget_grants(a.budget, r);
        int32_t s = 0, id = -1;
        if (go && listed) {
            id = take_listed(a.v, a.free_list, (long long)r);   // request r takes the r-th free page
            s = 1;
        }
        if (r >= a.n || id >= 0) {
            // past the last request, or served from the list
        } else if (!go) {
            // past the launch budget: no free page is left for this request
        } else if constexpr (K == Walk::Page) {
            const int32_t seed0 = request_seed(a.seed, r);
            id = walk_page(a.v, seed0, a.max_steps, &s);
        } else if constexpr (K == Walk::Word32) {
            const int32_t seed0 = request_seed(a.seed, r);
            id = walk_word<uint32_t>(a.v, seed0, a.max_steps, &s);
        } else if constexpr (K == Walk::Word64) {
            const int32_t seed0 = request_seed(a.seed, r);
            id = walk_word<uint64_t>(a.v, seed0, a.max_steps, &s);
        } else if constexpr (K == Walk::Crw) {
            const int32_t seed0 = request_seed(a.seed, r);
            int32_t* cur = a.cursors + (r % a.max_slots);
            int32_t c = *cur;
            id = walk_crw(a.v, &c, seed0, a.max_steps, &s);
            *cur = c;
        } else if constexpr (K == Walk::SingleClock) {
            id = sweep_single(a.v, a.arm, a.max_steps, &s);
        } else {
            uint32_t* arm = a.arms + (r % a.max_slots);
            uint32_t ar = *arm;
            id = sweep_dist(a.v, &ar, a.max_steps, &s);
            *arm = ar;
        }
        if (r >= a.n) continue;
        a.ids[r] = id;
        if (a.steps) a.steps[r] = s;
        acc.ok += id >= 0;
        acc.fail += id < 0;
        acc.steps += (unsigned long long)s;
    }
    flush_acc(acc, a.stats);
}

// Warp-collaborative walk: groups of W lanes take W consecutive requests.
// Launched with blockDim a multiple of W (>= W); a one-group launch
// (blockDim == W, one block) replays the groups in request order.
template <int W, typename Word>
__global__ void __launch_bounds__(256) k_alloc_collab(AllocArgs a) {
    __shared__ int32_t slots[256];
    Acc acc;
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t nthr = (uint64_t)gridDim.x * blockDim.x;
    const uint32_t gl = threadIdx.x & (uint32_t)(W - 1);
    const uint32_t L = WordTraits<Word>::count(a.v);
    const uint32_t lane_off = (uint32_t)(((unsigned long long)gl * a.stride) % L);
    volatile int32_t* my_slots = slots + (threadIdx.x & ~(uint32_t)(W - 1));
    const bool listed = a.budget && __ldcg(&a.budget->list_mode);
    // trip count uniform across each group of W lanes
    for (uint64_t base = tid - gl; base < a.n; base += nthr) {
        const uint64_t r = base + gl;
        const bool need = r < a.n && budget_grants(a.budget, r);
        const int32_t from_list = (need && listed) ? take_listed(a.v, a.free_list, (long long)r) : -1;
        int32_t s = 0;
        int32_t id = walk_collab<W, Word>(a.v, need && from_list < 0, request_seed(a.seed, base), lane_off,
                                          a.dedupe != 0, a.max_steps, my_slots, &s);
        if (from_list >= 0) {
            id = from_list;
            s = 1;
        }
        if (r < a.n) {
            a.ids[r] = id;
            if (a.steps) a.steps[r] = need ? s : 0;   // refused by the budget: no walk
            acc.ok += id >= 0;
            acc.fail += id < 0;
            acc.steps += (unsigned long long)s;
        }
    }
    flush_acc(acc, a.stats);
}

__global__ void __launch_bounds__(256) k_fifo_alloc(AllocArgs a, FifoState* st, int32_t* ring) {
    Acc acc;
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t nthr = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t r = tid; r < a.n; r += nthr) {
        int32_t s = 0;
        int32_t id = fifo_get(a.v, st, ring, a.stats, &s);
        a.ids[r] = id;
        if (a.steps) a.steps[r] = s;
        acc.ok += id >= 0;
        acc.fail += id < 0;
        acc.steps += (unsigned long long)s;
    }
    flush_acc(acc, a.stats);
}

__global__ void __launch_bounds__(256) k_fifo_free(PoolView v, uint32_t n, const int32_t* ids,
                                                   FifoState* st, int32_t* ring, DevStats* stats) {
    unsigned long long f = 0;
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (uint64_t)gridDim.x * blockDim.x) {
        int32_t id = ids[r];
        if (id < 0 || (uint32_t)id >= v.n_pages) continue;
        if (fifo_put(v, st, ring, stats, id)) ++f;
    }
    block_add_counters<1>({f}, {&stats->frees});
}

// ---- frees ----
__global__ void __launch_bounds__(256) k_free_pages(PoolView v, uint32_t n, const int32_t* ids,
                                                    int merge, DevStats* stats) {
    unsigned long long f = 0;
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t nthr = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t n_round = ((uint64_t)n + 31u) & ~31ull;
    for (uint64_t r = tid; r < n_round; r += nthr) {
        int32_t id = r < n ? ids[r] : -1;
        if (id >= (int32_t)v.n_pages) id = -1;
        if (merge && blockDim.x >= 32) {
            free_page_warp(v, 0xffffffffu, id);
        } else if (id >= 0) {
            free_page(v, id);
        }
        f += id >= 0;
    }
    block_add_counters<1>({f}, {&stats->frees});
}

// ---- contiguous runs ----
// SPAN: runs may cross word boundaries (1 <= k <= kMaxSpanPages); else one
// word holds the run (1 <= k <= 32, the reference's getXPage semantics).
template <bool SPAN>
__global__ void __launch_bounds__(256) k_alloc_runs(AllocArgs a, const int32_t* npages) {
    Acc acc;
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < a.n; r += (uint64_t)gridDim.x * blockDim.x) {
        int32_t k = npages[r];
        int32_t s = 0, id = -1;
        if (SPAN) {
            if (k >= 1 && (uint32_t)k <= kMaxSpanPages)
                id = walk_span(a.v, (uint32_t)k, request_seed(a.seed, r), a.max_steps, &s);
        } else if (k >= 1 && k <= 32) {
            id = walk_run(a.v, (uint32_t)k, request_seed(a.seed, r), a.max_steps, &s);
        }
        a.ids[r] = id;
        if (a.steps) a.steps[r] = s;
        acc.ok += id >= 0;
        acc.fail += id < 0;
        acc.steps += (unsigned long long)s;
    }
    flush_acc(acc, a.stats);
}

__global__ void __launch_bounds__(256) k_free_runs(PoolView v, uint32_t n, const int32_t* ids,
                                                   const int32_t* npages, DevStats* stats) {
    unsigned long long f = 0;
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (uint64_t)gridDim.x * blockDim.x) {
        int32_t id = ids[r], k = npages[r];
        if (id < 0 || k < 1 || (uint32_t)k > kMaxSpanPages || (unsigned long long)id + (uint32_t)k > v.n_pages)
            continue;
        free_span(v, id, (uint32_t)k);
        f += (unsigned long long)k;
    }
    block_add_counters<1>({f}, {&stats->frees});
}

// ---- config-1 step: claim one page, write the payload, free ----
// Each request claims a page with the page-probe walk, writes its request
// index into every 4-byte word of the first payload_words words of the page,
// and frees the page unless `hold` (unitTest1.5.cu:138-150 get/free kernels
// plus the payload write of the page-pool workload).
__global__ void __launch_bounds__(256) k_claim_write_free(AllocArgs a, uint32_t payload_words, int hold) {
    Acc acc;
    unsigned long long frees = 0;
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < a.n; r += (uint64_t)gridDim.x * blockDim.x) {
        int32_t s = 0;
        int32_t id = walk_page(a.v, request_seed(a.seed, r), a.max_steps, &s);
        a.ids[r] = id;
        if (a.steps) a.steps[r] = s;
        if (id >= 0) {
            int32_t* pg = reinterpret_cast<int32_t*>(a.v.base + (size_t)(uint32_t)id * a.v.page_size);
            uint32_t k = 0;
            if (((a.v.page_size | (uint32_t)(uintptr_t)a.v.base) & 15u) == 0u) {   // 16-byte aligned pages: 16 bytes a store
                const int4 v4 = make_int4((int32_t)r, (int32_t)r, (int32_t)r, (int32_t)r);
                for (; k + 4u <= payload_words; k += 4u) *reinterpret_cast<int4*>(pg + k) = v4;
            }
            for (; k < payload_words; ++k) pg[k] = (int32_t)r;
            if (!hold) { free_page(a.v, id); ++frees; }
        }
        acc.ok += id >= 0;
        acc.fail += id < 0;
        acc.steps += (unsigned long long)s;
    }
    block_add_counters<4>({acc.ok, acc.fail, acc.steps, frees},
                          {&a.stats->successes, &a.stats->failures, &a.stats->steps, &a.stats->frees});
}

__global__ void k_gather_pages(PoolView v, const int32_t* ids, uint32_t n, uint32_t words_per_page,
                               int32_t* out) {
    const unsigned long long total = (unsigned long long)n * words_per_page;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        uint32_t r = (uint32_t)(i / words_per_page), k = (uint32_t)(i % words_per_page);
        int32_t id = ids[r];
        out[i] = (id >= 0 && (uint32_t)id < v.n_pages)
                     ? reinterpret_cast<const int32_t*>(v.base + (size_t)(uint32_t)id * v.page_size)[k]
                     : 0;
    }
}

}  // namespace pbm

using namespace pbm;

namespace {

int check_cfg(const pbm_walk_config* c) {
    if (!c) return PBM_ERR_INVALID;
    if (c->strategy < 0 || c->strategy >= PBM_N_STRATEGIES) return PBM_ERR_INVALID;
    if (c->word_bits != 0 && c->word_bits != 32 && c->word_bits != 64) return PBM_ERR_INVALID;
    if (c->collab_width != 0 && c->collab_width != 8 && c->collab_width != 16 && c->collab_width != 32)
        return PBM_ERR_INVALID;
    if (c->block_size < 0 || c->block_size > 1024 || (c->block_size % 32) != 0) return PBM_ERR_INVALID;
    return PBM_OK;
}

AllocArgs make_args(pbm_pool* p, const pbm_walk_config* c, uint32_t n, uint32_t seed, int32_t* ids,
                    int32_t* steps) {
    AllocArgs a;
    a.v = p->view;
    a.n = n;
    a.seed = seed;
    a.max_steps = c->max_steps ? c->max_steps : kDefaultMaxSteps;
    a.stride = c->stride ? c->stride : 1u;
    a.ids = ids;
    a.steps = steps;
    a.stats = p->d_stats;
    a.cursors = p->d_cursors;
    a.arms = p->d_arms;
    a.arm = p->d_arm;
    a.max_slots = p->max_slots;
    int W = c->collab_width ? c->collab_width : 32;
    uint32_t L = c->word_bits == 64 ? p->view.n_words64 : p->view.n_words32;
    a.dedupe = ((unsigned long long)(W - 1) * a.stride >= L) ? 1 : 0;
    a.budget = nullptr;
    a.free_list = nullptr;
    return a;
}

template <int W, typename Word>
int launch_collab_w(const AllocArgs& a, int grid, int block, cudaStream_t s) {
    k_alloc_collab<W, Word><<<grid, block, 0, s>>>(a);
    PBM_LAUNCH_CHECK();
    return PBM_OK;
}

int launch_alloc(pbm_pool* p, const pbm_walk_config* c, const AllocArgs& a, bool serial,
                 cudaStream_t s) {
    const int block_cfg = c->block_size ? c->block_size : kDefaultBlock;
    const int W = c->collab_width ? c->collab_width : 32;
    const bool w64 = c->word_bits == 64;
    int block = serial ? 1 : block_cfg;
    int grid = serial ? 1 : (int)((a.n + (uint32_t)block - 1u) / (uint32_t)block);
    if (grid < 1) grid = 1;
    switch (c->strategy) {
    case PBM_RANDOM_WALK:
        k_alloc_thread<Walk::Page><<<grid, block, 0, s>>>(a);
        break;
    case PBM_RANDOM_WALK_BM:
        if (w64) k_alloc_thread<Walk::Word64><<<grid, block, 0, s>>>(a);
        else k_alloc_thread<Walk::Word32><<<grid, block, 0, s>>>(a);
        break;
    case PBM_CLUSTERED_RW_BM:
        k_alloc_thread<Walk::Crw><<<grid, block, 0, s>>>(a);
        break;
    case PBM_SINGLE_CLOCK:
        k_alloc_thread<Walk::SingleClock><<<grid, block, 0, s>>>(a);
        break;
    case PBM_DIST_CLOCK:
        k_alloc_thread<Walk::DistClock><<<grid, block, 0, s>>>(a);
        break;
    case PBM_COLLAB_RW_BM: {
        int cb = serial ? W : block_cfg;
        int cg = serial ? 1 : (int)((a.n + (uint32_t)cb - 1u) / (uint32_t)cb);
        if (cg < 1) cg = 1;
        if (W == 8) return w64 ? launch_collab_w<8, uint64_t>(a, cg, cb, s) : launch_collab_w<8, uint32_t>(a, cg, cb, s);
        if (W == 16) return w64 ? launch_collab_w<16, uint64_t>(a, cg, cb, s) : launch_collab_w<16, uint32_t>(a, cg, cb, s);
        return w64 ? launch_collab_w<32, uint64_t>(a, cg, cb, s) : launch_collab_w<32, uint32_t>(a, cg, cb, s);
    }
    case PBM_LINKED_LIST: {
        if (!p->fifo_valid) {
            int rc = fifo_build(p, s);
            if (rc) return rc;
        }
        k_fifo_alloc<<<grid, block, 0, s>>>(a, p->d_fifo, p->d_ring);
        break;
    }
    default:
        return PBM_ERR_INVALID;
    }
    PBM_LAUNCH_CHECK();
    return PBM_OK;
}

}  // namespace

extern "C" {

int pbm_alloc(pbm_pool* pool, const pbm_walk_config* cfg, uint32_t n, uint32_t seed, int32_t* d_ids,
              int32_t* d_steps, void* stream) {
    PBM_ON_POOL_DEVICE(pool);
    if (!pool || (n && !d_ids)) return PBM_ERR_INVALID;
    int rc = check_cfg(cfg);
    if (rc) return rc;
    if (n == 0) return PBM_OK;
    AllocArgs a = make_args(pool, cfg, n, seed, d_ids, d_steps);
    if (cfg->strategy != PBM_LINKED_LIST) pool->fifo_valid = false;
    if (cfg->fail_fast && cfg->strategy != PBM_LINKED_LIST) {   // the free list counts its pages itself
        rc = budget_prepare(pool, n, (cudaStream_t)stream);
        if (rc) return rc;
        a.budget = pool->d_budget;
        a.free_list = pool->d_free_list;
    }
    return launch_alloc(pool, cfg, a, false, (cudaStream_t)stream);
}

int pbm_alloc_serial(pbm_pool* pool, const pbm_walk_config* cfg, uint32_t n, uint32_t seed,
                     int32_t* d_ids, int32_t* d_steps, void* stream) {
    PBM_ON_POOL_DEVICE(pool);
    if (!pool || (n && !d_ids)) return PBM_ERR_INVALID;
    int rc = check_cfg(cfg);
    if (rc) return rc;
    if (n == 0) return PBM_OK;
    AllocArgs a = make_args(pool, cfg, n, seed, d_ids, d_steps);
    if (cfg->strategy != PBM_LINKED_LIST) pool->fifo_valid = false;
    return launch_alloc(pool, cfg, a, true, (cudaStream_t)stream);
}

int pbm_free(pbm_pool* pool, const pbm_walk_config* cfg, uint32_t n, const int32_t* d_ids, void* stream) {
    PBM_ON_POOL_DEVICE(pool);
    if (!pool || (n && !d_ids)) return PBM_ERR_INVALID;
    int rc = check_cfg(cfg);
    if (rc) return rc;
    if (n == 0) return PBM_OK;
    cudaStream_t s = (cudaStream_t)stream;
    int block = cfg->block_size ? cfg->block_size : kDefaultBlock;
    int grid = (int)((n + (uint32_t)block - 1u) / (uint32_t)block);
    if (cfg->strategy == PBM_LINKED_LIST) {
        if (!pool->fifo_valid) {
            rc = fifo_build(pool, s);
            if (rc) return rc;
        }
        k_fifo_free<<<grid, block, 0, s>>>(pool->view, n, d_ids, pool->d_fifo, pool->d_ring, pool->d_stats);
    } else {
        pool->fifo_valid = false;
        k_free_pages<<<grid, block, 0, s>>>(pool->view, n, d_ids, cfg->free_merge, pool->d_stats);
    }
    PBM_LAUNCH_CHECK();
    return PBM_OK;
}

static int alloc_runs_impl(pbm_pool* pool, uint32_t n, const int32_t* d_npages, uint32_t seed,
                           uint32_t max_steps, int32_t* d_ids, int32_t* d_steps, bool serial,
                           bool span, void* stream) {
    if (!pool || (n && (!d_ids || !d_npages))) return PBM_ERR_INVALID;
    if (n == 0) return PBM_OK;
    pbm_walk_config c{};
    c.strategy = PBM_RANDOM_WALK_BM;
    c.max_steps = max_steps;
    AllocArgs a = make_args(pool, &c, n, seed, d_ids, d_steps);
    int block = serial ? 1 : kDefaultBlock;
    int grid = serial ? 1 : (int)((n + (uint32_t)block - 1u) / (uint32_t)block);
    if (span) k_alloc_runs<true><<<grid, block, 0, (cudaStream_t)stream>>>(a, d_npages);
    else k_alloc_runs<false><<<grid, block, 0, (cudaStream_t)stream>>>(a, d_npages);
    PBM_LAUNCH_CHECK();
    pool->fifo_valid = false;
    return PBM_OK;
}

int pbm_alloc_runs(pbm_pool* pool, uint32_t n, const int32_t* d_npages, uint32_t seed,
                   uint32_t max_steps, int32_t* d_ids, int32_t* d_steps, void* stream) {
    PBM_ON_POOL_DEVICE(pool);
    return alloc_runs_impl(pool, n, d_npages, seed, max_steps, d_ids, d_steps, false, false, stream);
}

int pbm_alloc_runs_serial(pbm_pool* pool, uint32_t n, const int32_t* d_npages, uint32_t seed,
                          uint32_t max_steps, int32_t* d_ids, int32_t* d_steps, void* stream) {
    PBM_ON_POOL_DEVICE(pool);
    return alloc_runs_impl(pool, n, d_npages, seed, max_steps, d_ids, d_steps, true, false, stream);
}

int pbm_alloc_spans(pbm_pool* pool, uint32_t n, const int32_t* d_npages, uint32_t seed,
                    uint32_t max_steps, int32_t* d_ids, int32_t* d_steps, void* stream) {
    PBM_ON_POOL_DEVICE(pool);
    return alloc_runs_impl(pool, n, d_npages, seed, max_steps, d_ids, d_steps, false, true, stream);
}

int pbm_alloc_spans_serial(pbm_pool* pool, uint32_t n, const int32_t* d_npages, uint32_t seed,
                           uint32_t max_steps, int32_t* d_ids, int32_t* d_steps, void* stream) {
    PBM_ON_POOL_DEVICE(pool);
    return alloc_runs_impl(pool, n, d_npages, seed, max_steps, d_ids, d_steps, true, true, stream);
}

int pbm_free_runs(pbm_pool* pool, uint32_t n, const int32_t* d_ids, const int32_t* d_npages, void* stream) {
    PBM_ON_POOL_DEVICE(pool);
    if (!pool || (n && (!d_ids || !d_npages))) return PBM_ERR_INVALID;
    if (n == 0) return PBM_OK;
    int grid = (int)((n + 255u) / 256u);
    k_free_runs<<<grid, 256, 0, (cudaStream_t)stream>>>(pool->view, n, d_ids, d_npages, pool->d_stats);
    PBM_LAUNCH_CHECK();
    pool->fifo_valid = false;
    return PBM_OK;
}

int pbm_claim_write_free(pbm_pool* pool, uint32_t n, uint32_t seed, uint32_t payload_bytes, int hold,
                         uint32_t max_steps, int32_t* d_ids, int32_t* d_steps, void* stream) {
    PBM_ON_POOL_DEVICE(pool);
    if (!pool || (n && !d_ids) || !pool->d_base || payload_bytes > pool->page_size || (payload_bytes & 3u))
        return PBM_ERR_INVALID;
    if (n == 0) return PBM_OK;
    pbm_walk_config c{};
    c.strategy = PBM_RANDOM_WALK;
    c.max_steps = max_steps;
    AllocArgs a = make_args(pool, &c, n, seed, d_ids, d_steps);
    // a batch too small to give every SM two 256-thread blocks runs in
    // 64-thread blocks, so its walks spread over every SM
    const int block = n < (uint32_t)sm_count() * 512u ? 64 : 256;
    int grid = (int)((n + (uint32_t)block - 1u) / (uint32_t)block);
    k_claim_write_free<<<grid, block, 0, (cudaStream_t)stream>>>(a, payload_bytes / 4u, hold);
    PBM_LAUNCH_CHECK();
    pool->fifo_valid = false;
    return PBM_OK;
}

int pbm_gather_pages(pbm_pool* pool, const int32_t* d_ids, uint32_t n, uint32_t bytes_per_page,
                     int32_t* d_out, void* stream) {
    PBM_ON_POOL_DEVICE(pool);
    if (!pool || !pool->d_base || (n && (!d_ids || !d_out)) || bytes_per_page > pool->page_size ||
        (bytes_per_page & 3u) || bytes_per_page == 0)
        return PBM_ERR_INVALID;
    if (n == 0) return PBM_OK;
    k_gather_pages<<<sm_count() * 4, 256, 0, (cudaStream_t)stream>>>(pool->view, d_ids, n, bytes_per_page / 4u,
                                                                     d_out);
    PBM_LAUNCH_CHECK();
    return PBM_OK;
}

}  // extern "C"
