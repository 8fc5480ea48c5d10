// malloc.cu -- batched size-classed malloc / free over a pool's pages, with
// two backends: page runs with live counts (pbm/pbm_malloc.cuh) and per-class
// block queues (pbm/pbm_qmalloc.cuh).  Forms: plain (one launch per group),
// persistent (one launch), a one-warp deterministic replay, and the
// CUDA-graph form.
//
// Reference: mallocRW / freeRW (source/RWMalloc.cuh:299-334), the
// KernelMallocCollab allocator (source/malloc.cu:223-320) and the
// malloc/free drivers (unitTests/unitTest3.cu, unitTestMalloc1.cu).
#include <mutex>
#include <new>

#include "batch_common.cuh"
#include "pbm/pbm_malloc.cuh"
#include "pbm/pbm_qmalloc.cuh"

namespace pbm {
namespace {

struct MArgs {
    MallocView m;
    QMallocView qm;
    const pbm_group* groups;
    uint32_t n_groups;
    const uint32_t* d_step;
    uint32_t n_steps;                 // graph form: replay k uses descriptor table k mod n_steps
    uint32_t seed;
    const uint32_t* sizes;            // per slot
    unsigned long long* ptrs;         // per slot (device addresses, 0 = none)
    unsigned long long arena_len;
    const unsigned long long* prefix;
    uint32_t max_steps;
    DevStats* stats;
    int32_t op;                       // plain form: the one group this launch serves
    uint32_t count;
    unsigned long long offset;
    unsigned long long q_base;
};

struct MAcc {
    unsigned long long ok = 0, fail = 0, steps = 0, frees = 0, bad = 0;
};

__device__ __forceinline__ unsigned long long wrap(unsigned long long slot, unsigned long long len) {
    if (slot >= len) slot = slot - len < len ? slot - len : slot % len;
    return slot;
}

// Q: the queue backend (pbm_qmalloc.cuh), else page runs (pbm_malloc.cuh).
template <bool SERIAL, bool Q>
__device__ __forceinline__ void malloc_round(const MArgs& a, uint32_t seed, bool active, int op,
                                             unsigned long long q0, unsigned long long q,
                                             unsigned long long slot, MAcc& acc) {
    const bool do_malloc = active && op == PBM_OP_MALLOC;
    const bool do_free = active && op == PBM_OP_MFREE;
    const uint64_t size = do_malloc ? (uint64_t)a.sizes[slot] : 0ull;
    int32_t s = 0;
    void* p;
    if constexpr (Q) {
        p = qmalloc_group(a.qm, 0xffffffffu, size, request_seed(seed, (uint32_t)q), a.max_steps, SERIAL, &s);
    } else {
        p = malloc_group(a.m, 0xffffffffu, size, request_seed(seed ^ 0x9E3779B9u, (uint32_t)q0),
                         request_seed(seed, (uint32_t)q), a.max_steps, SERIAL, &s);
    }
    if (do_malloc) {
        a.ptrs[slot] = (unsigned long long)p;
        if (size) {
            acc.ok += p != nullptr;
            acc.fail += p == nullptr;
            acc.steps += (unsigned long long)s;
        }
    }
    const void* fp = do_free ? (const void*)a.ptrs[slot] : nullptr;
    bool ok;
    if constexpr (Q) ok = qfree_group(a.qm, 0xffffffffu, fp);
    else ok = free_group(a.m, 0xffffffffu, fp);
    if (do_free) {
        a.ptrs[slot] = 0ull;
        if (fp) {
            acc.frees += ok;
            acc.bad += !ok;
        }
    }
}

__device__ __forceinline__ void flush_macc(const MAcc& c, DevStats* st) {
    block_add_counters<5>({c.ok, c.fail, c.steps, c.frees, c.bad},
                          {&st->successes, &st->failures, &st->steps, &st->frees, &st->bad_frees});
}

template <bool SERIAL, bool Q>
__global__ void __launch_bounds__(256) k_malloc_persistent(MArgs a) {
    MAcc acc;
    const uint32_t step = a.d_step ? *a.d_step : 0u;
    const pbm_group* groups = a.groups + (a.d_step ? (size_t)(step % a.n_steps) * a.n_groups : 0);
    const uint32_t seed = a.seed + step;
    const unsigned long long total = a.prefix[a.n_groups];
    const uint32_t lane = threadIdx.x & 31u;
    const unsigned long long warp0 = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned long long nwarps = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
    for (unsigned long long chunk = warp0; chunk * 32ull < total; chunk += nwarps) {
        const unsigned long long q0 = chunk * 32ull;
        const unsigned long long q = q0 + lane;
        const bool active = q < total;
        uint32_t g0 = 0;
        if (lane == 0) g0 = find_group(a.prefix, a.n_groups, q0, 0u);
        g0 = __shfl_sync(0xffffffffu, g0, 0);
        const unsigned long long g0_end = __ldg(a.prefix + g0 + 1u);
        int op = PBM_OP_MALLOC;
        unsigned long long slot = 0;
        if (active) {
            const uint32_t g = q < g0_end ? g0 : find_group(a.prefix, a.n_groups, q, g0);
            const pbm_group gd = groups[g];
            op = gd.op;
            slot = wrap(gd.offset + (q - __ldg(a.prefix + g)), a.arena_len);
        }
        malloc_round<SERIAL, Q>(a, seed, active, op, q0, q, slot, acc);
    }
    flush_macc(acc, a.stats);
}

template <bool Q>
__global__ void __launch_bounds__(256) k_malloc_plain(MArgs a) {
    MAcc acc;
    const uint32_t lane = threadIdx.x & 31u;
    const unsigned long long warp0 = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned long long nwarps = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
    for (unsigned long long chunk = warp0; chunk * 32ull < a.count; chunk += nwarps) {
        const unsigned long long ql = chunk * 32ull + lane;
        const bool active = ql < a.count;
        malloc_round<false, Q>(a, a.seed, active, a.op, a.q_base + chunk * 32ull, a.q_base + ql,
                            wrap(a.offset + ql, a.arena_len), acc);
    }
    flush_macc(acc, a.stats);
}

__global__ void k_malloc_init(int32_t* start_of, int32_t* live, uint8_t* len_of, uint32_t n) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        start_of[i] = -1;
        live[i] = 0;
        len_of[i] = 0;
    }
}

struct MallocTables {
    // page-run backend
    int32_t* start_of = nullptr;
    int32_t* live = nullptr;
    uint8_t* len_of = nullptr;
    // queue backend
    QueueRing* rings = nullptr;
    uint32_t* slots = nullptr;
    uint8_t* class_of = nullptr;
    unsigned long long* qcounters = nullptr;
    uint32_t qcap = 0;
    // shared
    unsigned long long* prefix = nullptr;
    uint32_t prefix_cap = 0;
};

__global__ void k_qmalloc_init(QueueRing* rings, uint32_t capacity) {
    const int c = threadIdx.x;
    if (c < kQClasses) {
        rings[c].head = rings[c].tail = rings[c].avail = 0ull;
        rings[c].space = capacity;
    }
}

}  // namespace
}  // namespace pbm

using namespace pbm;

namespace {

// Malloc tables of a pool live beside it, keyed by the pool handle.  Every
// entry point takes g_reg_mu for its whole call (launches only enqueue work),
// so tables are never moved or freed under another thread's call.
std::mutex g_reg_mu;
struct Registry {
    pbm_pool* pool;
    MallocTables t;
};
Registry g_reg[64];
int g_nreg = 0;

MallocTables* tables_of(pbm_pool* p) {
    for (int i = 0; i < g_nreg; ++i) if (g_reg[i].pool == p) return &g_reg[i].t;
    return nullptr;
}

MallocTables* tables_add(pbm_pool* p) {
    if (MallocTables* t = tables_of(p)) return t;
    if (g_nreg >= 64) return nullptr;
    g_reg[g_nreg].pool = p;
    g_reg[g_nreg].t = MallocTables{};
    return &g_reg[g_nreg++].t;
}

uint32_t page_shift_of(const pbm_pool* p) {
    uint32_t sh = 0;
    while ((1u << sh) < p->page_size) ++sh;
    return sh;
}

MallocView view_of(pbm_pool* p, const MallocTables* t) {
    MallocView m;
    m.pool = p->view;
    m.start_of = t->start_of;
    m.live = t->live;
    m.len_of = t->len_of;
    m.page_shift = page_shift_of(p);
    return m;
}

QMallocView qview_of(pbm_pool* p, const MallocTables* t) {
    QMallocView q;
    q.pool = p->view;
    q.rings = t->rings;
    q.slots = t->slots;
    q.class_of = t->class_of;
    q.counters = t->qcounters;
    q.capacity = t->qcap;
    q.page_shift = page_shift_of(p);
    return q;
}

int check_pool(pbm_pool* p) {
    if (!p || !p->d_base) return PBM_ERR_INVALID;
    if ((p->page_size & (p->page_size - 1u)) || p->page_size < 2048u || p->page_size > (1u << 16))
        return PBM_ERR_INVALID;
    return PBM_OK;
}

void free_queue(MallocTables* t) {
    cudaFree(t->rings);
    cudaFree(t->slots);
    cudaFree(t->class_of);
    cudaFree(t->qcounters);
    t->rings = nullptr;
    t->slots = nullptr;
    t->class_of = nullptr;
    t->qcounters = nullptr;
    t->qcap = 0;
}

void drop_if_empty(pbm_pool* p) {
    for (int i = 0; i < g_nreg; ++i) {
        if (g_reg[i].pool != p) continue;
        MallocTables& t = g_reg[i].t;
        if (!t.start_of && !t.rings) {
            cudaFree(t.prefix);
            g_reg[i] = g_reg[--g_nreg];
        }
        return;
    }
}

bool ensure_prefix(MallocTables* t, uint32_t n_groups) {
    if (t->prefix_cap >= n_groups + 1u) return true;
    cudaFree(t->prefix);
    t->prefix = nullptr;
    if (cudaMalloc(&t->prefix, sizeof(unsigned long long) * (n_groups + 1u)) != cudaSuccess) {
        cudaGetLastError();
        t->prefix_cap = 0;
        return false;
    }
    t->prefix_cap = n_groups + 1u;
    return true;
}

template <bool Q>
int persistent_blocks() {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_malloc_persistent<false, Q>, 256, 0);
    return per_sm < 1 ? 1 : per_sm;
}

int batch_impl(pbm_pool* pool, bool queue, const pbm_group* d_groups, const pbm_group* h_groups, uint32_t n_groups,
               const uint32_t* d_sizes, unsigned long long* d_ptrs, uint64_t arena_len, uint32_t seed,
               uint32_t max_steps, int mode, void* stream) {
    MallocTables* t = tables_of(pool);
    if (!t || (queue ? !t->rings : !t->start_of) || !d_ptrs || !arena_len) return PBM_ERR_INVALID;
    if (n_groups == 0) return PBM_OK;
    cudaStream_t s = (cudaStream_t)stream;
    pool->fifo_valid = false;
    MArgs a{};
    if (queue) a.qm = qview_of(pool, t);
    else a.m = view_of(pool, t);
    a.seed = seed;
    a.sizes = d_sizes;
    a.ptrs = d_ptrs;
    a.arena_len = arena_len;
    a.max_steps = max_steps ? max_steps : kDefaultMaxSteps;
    a.stats = pool->d_stats;
    if (mode == PBM_LAUNCH_PLAIN) {
        if (!h_groups) return PBM_ERR_INVALID;
        unsigned long long q = 0;
        for (uint32_t g = 0; g < n_groups; ++g) {
            const pbm_group& gd = h_groups[g];
            if (gd.op != PBM_OP_MALLOC && gd.op != PBM_OP_MFREE) return PBM_ERR_INVALID;
            if (gd.count == 0) continue;
            a.op = gd.op;
            a.count = gd.count;
            a.offset = gd.offset;
            a.q_base = q;
            const unsigned long long warps = (gd.count + 31ull) / 32ull;
            const unsigned grid = (unsigned)((warps * 32ull + 255ull) / 256ull);
            if (queue) k_malloc_plain<true><<<grid, 256, 0, s>>>(a);
            else k_malloc_plain<false><<<grid, 256, 0, s>>>(a);
            PBM_LAUNCH_CHECK();
            q += gd.count;
        }
        return PBM_OK;
    }
    if ((mode != PBM_LAUNCH_PERSISTENT && mode != PBM_LAUNCH_SERIAL) || !d_groups) return PBM_ERR_INVALID;
    if (!ensure_prefix(t, n_groups)) return PBM_ERR_NOMEM;
    k_batch_prefix<<<1, 1024, 0, s>>>(d_groups, n_groups, nullptr, 0u, 1u, t->prefix);
    PBM_LAUNCH_CHECK();
    a.groups = d_groups;
    a.n_groups = n_groups;
    a.prefix = t->prefix;
    if (mode == PBM_LAUNCH_SERIAL) {
        if (queue) k_malloc_persistent<true, true><<<1, 32, 0, s>>>(a);
        else k_malloc_persistent<true, false><<<1, 32, 0, s>>>(a);
    } else if (queue) {
        k_malloc_persistent<false, true><<<sm_count() * persistent_blocks<true>(), 256, 0, s>>>(a);
    } else {
        k_malloc_persistent<false, false><<<sm_count() * persistent_blocks<false>(), 256, 0, s>>>(a);
    }
    PBM_LAUNCH_CHECK();
    return PBM_OK;
}

int graph_impl(pbm_pool* pool, bool queue, const pbm_group* d_groups, uint32_t n_groups, uint32_t n_steps,
               const uint32_t* d_sizes, unsigned long long* d_ptrs, uint64_t arena_len, uint32_t seed0,
               uint32_t max_steps, void* stream, pbm_graph** out) {
    MallocTables* t = tables_of(pool);
    if (!t || (queue ? !t->rings : !t->start_of) || !d_groups || !d_ptrs || !out || !n_groups || !n_steps ||
        !arena_len)
        return PBM_ERR_INVALID;
    *out = nullptr;
    cudaStream_t s = (cudaStream_t)stream;
    pbm_graph* g = new (std::nothrow) pbm_graph();
    if (!g) return PBM_ERR_NOMEM;
    g->device = pool->device;
    g->graph = nullptr;
    g->exec = nullptr;
    if (cudaMalloc(&g->d_step, sizeof(uint32_t)) != cudaSuccess ||
        cudaMalloc(&g->d_prefix, sizeof(unsigned long long) * (n_groups + 1u)) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(g->d_step);
        delete g;
        return PBM_ERR_NOMEM;
    }
    PBM_CUDA_TRY(cudaMemsetAsync(g->d_step, 0, sizeof(uint32_t), s));
    PBM_CUDA_TRY(cudaStreamSynchronize(s));
    MArgs a{};
    if (queue) a.qm = qview_of(pool, t);
    else a.m = view_of(pool, t);
    a.groups = d_groups;
    a.n_groups = n_groups;
    a.d_step = g->d_step;
    a.n_steps = n_steps;
    a.seed = seed0;
    a.sizes = d_sizes;
    a.ptrs = d_ptrs;
    a.arena_len = arena_len;
    a.prefix = g->d_prefix;
    a.max_steps = max_steps ? max_steps : kDefaultMaxSteps;
    a.stats = pool->d_stats;
    const int per_sm = queue ? persistent_blocks<true>() : persistent_blocks<false>();
    cudaStream_t cap = nullptr;
    PBM_CUDA_TRY(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        k_batch_prefix<<<1, 1024, 0, cap>>>(d_groups, n_groups, g->d_step, 0u, n_steps, g->d_prefix);
        if (queue) k_malloc_persistent<false, true><<<sm_count() * per_sm, 256, 0, cap>>>(a);
        else k_malloc_persistent<false, false><<<sm_count() * per_sm, 256, 0, cap>>>(a);
        k_step_advance<<<1, 32, 0, cap>>>(g->d_step);
        cudaGraph_t graph = nullptr;
        e = cudaStreamEndCapture(cap, &graph);
        if (e == cudaSuccess) {
            g->graph = graph;
            e = cudaGraphInstantiate(&g->exec, graph, 0);
        }
    }
    cudaStreamDestroy(cap);
    if (e != cudaSuccess) {
        cudaGetLastError();
        if (g->graph) cudaGraphDestroy(g->graph);
        cudaFree(g->d_step);
        cudaFree(g->d_prefix);
        delete g;
        return PBM_ERR_CUDA;
    }
    g->launches_per_replay = 3;
    pool->fifo_valid = false;
    *out = g;
    return PBM_OK;
}

}  // namespace

extern "C" {

int pbm_malloc_init(pbm_pool* pool) {
    PBM_ON_POOL_DEVICE(pool);
    std::lock_guard<std::mutex> lk(g_reg_mu);
    int rc = check_pool(pool);
    if (rc) return rc;
    MallocTables* t = tables_add(pool);
    if (!t) return PBM_ERR_NOMEM;
    if (t->start_of) return PBM_OK;
    const size_t n = pool->n_pages;
    if (cudaMalloc(&t->start_of, n * 4) != cudaSuccess || cudaMalloc(&t->live, n * 4) != cudaSuccess ||
        cudaMalloc(&t->len_of, n) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(t->start_of);
        cudaFree(t->live);
        t->start_of = nullptr;
        t->live = nullptr;
        t->len_of = nullptr;
        drop_if_empty(pool);
        return PBM_ERR_NOMEM;
    }
    k_malloc_init<<<sm_count() * 4, 256>>>(t->start_of, t->live, t->len_of, (uint32_t)n);
    PBM_LAUNCH_CHECK();
    PBM_CUDA_TRY(cudaDeviceSynchronize());
    return PBM_OK;
}

int pbm_malloc_tables(pbm_pool* pool, void** d_start_of, void** d_live, void** d_len_of) {
    PBM_ON_POOL_DEVICE(pool);
    std::lock_guard<std::mutex> lk(g_reg_mu);
    MallocTables* t = tables_of(pool);
    if (!t || !t->start_of) return PBM_ERR_INVALID;
    if (d_start_of) *d_start_of = t->start_of;
    if (d_live) *d_live = t->live;
    if (d_len_of) *d_len_of = t->len_of;
    return PBM_OK;
}

int pbm_malloc_release(pbm_pool* pool) {
    PBM_ON_POOL_DEVICE(pool);
    std::lock_guard<std::mutex> lk(g_reg_mu);
    MallocTables* t = tables_of(pool);
    if (!t) return PBM_ERR_INVALID;
    cudaDeviceSynchronize();
    cudaFree(t->start_of);
    cudaFree(t->live);
    cudaFree(t->len_of);
    t->start_of = nullptr;
    t->live = nullptr;
    t->len_of = nullptr;
    free_queue(t);
    drop_if_empty(pool);
    return PBM_OK;
}

int pbm_malloc_batch(pbm_pool* pool, const pbm_group* d_groups, const pbm_group* h_groups, uint32_t n_groups,
                     const uint32_t* d_sizes, unsigned long long* d_ptrs, uint64_t arena_len, uint32_t seed,
                     uint32_t max_steps, int mode, void* stream) {
    PBM_ON_POOL_DEVICE(pool);
    std::lock_guard<std::mutex> lk(g_reg_mu);
    return batch_impl(pool, false, d_groups, h_groups, n_groups, d_sizes, d_ptrs, arena_len, seed, max_steps, mode,
                      stream);
}

int pbm_malloc_graph_create(pbm_pool* pool, const pbm_group* d_groups, uint32_t n_groups, uint32_t n_steps,
                            const uint32_t* d_sizes, unsigned long long* d_ptrs, uint64_t arena_len,
                            uint32_t seed0, uint32_t max_steps, void* stream, pbm_graph** out) {
    PBM_ON_POOL_DEVICE(pool);
    std::lock_guard<std::mutex> lk(g_reg_mu);
    return graph_impl(pool, false, d_groups, n_groups, n_steps, d_sizes, d_ptrs, arena_len, seed0, max_steps, stream,
                      out);
}

int pbm_malloc_counts(pbm_pool* pool, uint64_t* h_live_runs, uint64_t* h_bad_frees, void* stream) {
    PBM_ON_POOL_DEVICE(pool);
    std::lock_guard<std::mutex> lk(g_reg_mu);
    MallocTables* t = tables_of(pool);
    if (!t || !t->start_of) return PBM_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    DevStats d;
    PBM_CUDA_TRY(cudaMemcpyAsync(&d, pool->d_stats, sizeof(d), cudaMemcpyDeviceToHost, s));
    PBM_CUDA_TRY(cudaStreamSynchronize(s));
    if (h_bad_frees) *h_bad_frees = d.bad_frees;
    if (h_live_runs) {
        // runs still holding blocks: count first pages with live > 0 (host scan of a snapshot)
        const size_t n = pool->n_pages;
        int32_t* h = new (std::nothrow) int32_t[n];
        if (!h) return PBM_ERR_NOMEM;
        cudaError_t e = cudaMemcpy(h, t->live, n * 4, cudaMemcpyDeviceToHost);
        uint64_t c = 0;
        for (size_t i = 0; i < n; ++i) c += h[i] > 0;
        delete[] h;
        if (e != cudaSuccess) { cudaGetLastError(); return PBM_ERR_CUDA; }
        *h_live_runs = c;
    }
    return PBM_OK;
}

// ---- queue backend ----

int pbm_qmalloc_init(pbm_pool* pool, uint32_t ring_capacity) {
    PBM_ON_POOL_DEVICE(pool);
    std::lock_guard<std::mutex> lk(g_reg_mu);
    int rc = check_pool(pool);
    if (rc) return rc;
    if (pool->n_pages * (uint64_t)pool->page_size > (1ull << 36)) return PBM_ERR_INVALID;   // 32-bit handles of 16 B
    const uint32_t cap = ring_capacity ? ring_capacity : (1u << 20);
    if (cap & (cap - 1u)) return PBM_ERR_INVALID;
    MallocTables* t = tables_add(pool);
    if (!t) return PBM_ERR_NOMEM;
    if (t->rings) return t->qcap == cap ? PBM_OK : PBM_ERR_INVALID;
    const size_t n = pool->n_pages;
    if (cudaMalloc(&t->rings, sizeof(QueueRing) * kQClasses) != cudaSuccess ||
        cudaMalloc(&t->slots, sizeof(uint32_t) * (size_t)kQClasses * cap) != cudaSuccess ||
        cudaMalloc(&t->class_of, n) != cudaSuccess ||
        cudaMalloc(&t->qcounters, sizeof(unsigned long long) * kQCounterWords) != cudaSuccess) {
        cudaGetLastError();
        free_queue(t);
        drop_if_empty(pool);
        return PBM_ERR_NOMEM;
    }
    t->qcap = cap;
    PBM_CUDA_TRY(cudaMemset(t->slots, 0xff, sizeof(uint32_t) * (size_t)kQClasses * cap));
    PBM_CUDA_TRY(cudaMemset(t->class_of, 0, n));
    PBM_CUDA_TRY(cudaMemset(t->qcounters, 0, sizeof(unsigned long long) * kQCounterWords));
    k_qmalloc_init<<<1, 32>>>(t->rings, cap);
    PBM_LAUNCH_CHECK();
    PBM_CUDA_TRY(cudaDeviceSynchronize());
    return PBM_OK;
}

int pbm_qmalloc_release(pbm_pool* pool) {
    PBM_ON_POOL_DEVICE(pool);
    std::lock_guard<std::mutex> lk(g_reg_mu);
    MallocTables* t = tables_of(pool);
    if (!t || !t->rings) return PBM_ERR_INVALID;
    cudaDeviceSynchronize();
    free_queue(t);
    drop_if_empty(pool);
    return PBM_OK;
}

int pbm_qmalloc_batch(pbm_pool* pool, const pbm_group* d_groups, const pbm_group* h_groups, uint32_t n_groups,
                      const uint32_t* d_sizes, unsigned long long* d_ptrs, uint64_t arena_len, uint32_t seed,
                      uint32_t max_steps, int mode, void* stream) {
    PBM_ON_POOL_DEVICE(pool);
    std::lock_guard<std::mutex> lk(g_reg_mu);
    return batch_impl(pool, true, d_groups, h_groups, n_groups, d_sizes, d_ptrs, arena_len, seed, max_steps, mode,
                      stream);
}

int pbm_qmalloc_graph_create(pbm_pool* pool, const pbm_group* d_groups, uint32_t n_groups, uint32_t n_steps,
                             const uint32_t* d_sizes, unsigned long long* d_ptrs, uint64_t arena_len,
                             uint32_t seed0, uint32_t max_steps, void* stream, pbm_graph** out) {
    PBM_ON_POOL_DEVICE(pool);
    std::lock_guard<std::mutex> lk(g_reg_mu);
    return graph_impl(pool, true, d_groups, n_groups, n_steps, d_sizes, d_ptrs, arena_len, seed0, max_steps, stream,
                      out);
}

int pbm_qmalloc_counts(pbm_pool* pool, uint64_t* h_queued, uint64_t* h_chunks, uint64_t* h_overflow,
                       uint64_t* h_timeouts, uint64_t* h_bad_frees, void* stream) {
    PBM_ON_POOL_DEVICE(pool);
    std::lock_guard<std::mutex> lk(g_reg_mu);
    MallocTables* t = tables_of(pool);
    if (!t || !t->rings) return PBM_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    QueueRing r[kQClasses];
    unsigned long long c[kQCounterWords];
    PBM_CUDA_TRY(cudaMemcpyAsync(r, t->rings, sizeof(r), cudaMemcpyDeviceToHost, s));
    PBM_CUDA_TRY(cudaMemcpyAsync(c, t->qcounters, sizeof(c), cudaMemcpyDeviceToHost, s));
    PBM_CUDA_TRY(cudaStreamSynchronize(s));
    if (h_queued)
        for (int k = 0; k < kQClasses; ++k) h_queued[k] = (uint64_t)(long long)r[k].avail;
    if (h_chunks) *h_chunks = c[kQChunks];
    if (h_overflow) *h_overflow = c[kQOverflow];
    if (h_timeouts) *h_timeouts = c[kQTimeouts];
    if (h_bad_frees) *h_bad_frees = c[kQBadFrees];
    return PBM_OK;
}

}  // extern "C"
