// batch.cu -- batched alloc / free / swap requests from many caller groups.
//
// Requests of a batch are numbered in group order (q = 0 .. total-1) and
// request q always uses LCG seed request_seed(seed, q).  Three launch forms
// run the same requests:
//   plain       one kernel launch per group (what a caller gets by launching
//               its own kernel per batch, unitTest1.cu:64 style);
//   persistent  one kernel over all groups, a grid of (SMs x resident blocks);
//               each block scans the groups' counts into shared memory and
//               its warps pull 32-request chunks of the block's range from a
//               shared counter, finding a chunk's group by a ballot search of
//               the prefix sums;
//   graph       the persistent form captured once in a CUDA graph; the host
//               counts the replays and writes the step into the kernel's
//               parameters before each launch, so each replay is one launch
//               that reads the step's descriptors from device memory with no
//               counter to read first, and the last tenth of a step's chunks
//               sits in pools that blocks which finish their own range early
//               drain.
#include <atomic>
#include <new>
#include <cstring>
#include <type_traits>
#include <vector>

#include "batch_common.cuh"

namespace pbm {

// Collab2: the collaborative walk with two requests per lane (64 per warp),
// selected by collab_width 64.
enum class BWalk { Page, Word32, Word64, Collab, Collab2 };

template <BWalk K> constexpr int kReqPerLane = K == BWalk::Collab2 ? 2 : 1;

struct BatchArgs {
    PoolView v;
    const pbm_group* groups;            // base of the descriptor table
    uint32_t n_groups;
    uint32_t step;                      // graph form: the replay (set on the host before each launch)
    uint32_t n_steps;                   // descriptor tables (replay k uses table k mod n_steps; >= 1)
    uint32_t seed;
    int32_t* arena;
    unsigned long long arena_len;
    int32_t* steps;                     // parallel to arena, may be null
    int32_t* results;                   // per request q (request order), may be null or host-mapped
    const unsigned long long* prefix;   // persistent, not fused: n_groups + 1 exclusive prefix
    int32_t fuse;                       // persistent: each block scans the groups itself
    unsigned long long* pools;          // graph form: 2 x kPools tail-pool counters, 16 words apart (may be null)
    uint32_t max_steps;
    uint32_t stride;
    int32_t dedupe;
    int32_t merge;
    DevStats* stats;
    // plain form: the one group this launch serves
    int32_t op;
    uint32_t count;
    unsigned long long offset;
    unsigned long long q_base;
};

// The launch form may carry the step's descriptors in the kernel's parameter
// block (a host table of at most PBM_MAX_INLINE_GROUPS groups): the table then
// travels with the launch itself and a host-driven step needs no separate
// host-to-device copy.  NoTable is the empty parameter of the other forms.
struct GroupTable {
    pbm_group g[PBM_MAX_INLINE_GROUPS];
};
struct NoTable {};

// Per-thread counters of a launch; ok / fail / frees count requests of the
// thread (at most one per chunk it serves), steps may pass 2^32.
struct BAcc {
    uint32_t ok = 0, fail = 0, frees = 0;
    unsigned long long steps = 0;
};

__device__ __forceinline__ void flush_bacc(const BAcc& a, DevStats* st) {
    block_add_counters<4>({a.ok, a.fail, a.steps, a.frees},
                          {&st->successes, &st->failures, &st->steps, &st->frees});
}

// The persistent kernel's end, with no block barrier: each warp adds its
// sums into the block's shared counters (zeroed before the block's first
// barrier) and counts itself done; the last warp of the block adds the
// block's sums to the pool's counters.  Warps leave as soon as they are done.
__device__ __forceinline__ void flush_bacc_last_warp(const BAcc& a, DevStats* st, unsigned long long* s_acc,
                                                     unsigned int* s_warps_done) {
    const uint32_t lane = threadIdx.x & 31u;
    unsigned long long v[4] = {a.ok, a.fail, a.steps, a.frees};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], d);
    }
    unsigned int last = 0u;
    if (lane == 0u) {
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (v[k]) atomicAdd(s_acc + k, v[k]);
        __threadfence_block();
        last = atomicAdd(s_warps_done, 1u) == (blockDim.x >> 5) - 1u;
    }
    last = __shfl_sync(0xffffffffu, last, 0);
    if (last) {
        __threadfence_block();
        if (lane < 4u) {
            const unsigned long long x = atomicAdd(s_acc + lane, 0ull);   // every warp's sums
            unsigned long long* dst = lane == 0u ? &st->successes
                                    : lane == 1u ? &st->failures
                                    : lane == 2u ? &st->steps : &st->frees;
            if (x) atomicAdd(dst, x);
        }
    }
}

// The graph form's tail pools: the last 1/kPoolShare of a step's chunks,
// split into kPools ranges; block b drains pool b mod kPools once its own
// range is done.  Counters of replay k live at parity k & 1, so block 0 of
// replay k clears the parity replay k + 1 will use (replay k - 1 has
// finished with it).
constexpr uint32_t kPools = 8;
constexpr unsigned long long kPoolShare = 10;

// The request's result: arena update, counters, and the free of the page it
// gave up (merged per word within the warp when asked); converged call.
template <typename SlotT>
__device__ __forceinline__ void batch_finish(const BatchArgs& a, bool active, int op, unsigned long long q,
                                             SlotT slot, int32_t held, bool need, int32_t id, int32_t s,
                                             BAcc& acc) {
    int32_t to_free = -1;
    if (active) {
        if (a.results) a.results[q] = op == PBM_OP_FREE ? held : id;
        if (op == PBM_OP_ALLOC) {
            a.arena[slot] = id;
        } else if (op == PBM_OP_FREE) {
            to_free = held;
        } else if (id >= 0) {               // swap
            a.arena[slot] = id;
            to_free = held;
        }
        if (to_free >= (int32_t)a.v.n_pages) to_free = -1;
        if (need) {
            if (a.steps) a.steps[slot] = s;
            acc.ok += id >= 0;
            acc.fail += id < 0;
            acc.steps += (unsigned long long)s;
        }
        acc.frees += to_free >= 0;
    }
    if (a.merge) free_page_warp(a.v, 0xffffffffu, to_free);
    else if (to_free >= 0) free_page(a.v, to_free);
}

// One warp-wide round: every lane of the warp calls converged.
template <BWalk K, int W, typename Word>
__device__ __forceinline__ void batch_round(const BatchArgs& a, uint32_t seed, bool active, int op,
                                            unsigned long long q, unsigned long long slot,
                                            uint32_t lane_off, volatile int32_t* gslots, BAcc& acc) {
    const bool need = active && (op == PBM_OP_ALLOC || op == PBM_OP_SWAP);
    // the slot's held page is read before the walk so its latency overlaps it
    const int32_t held = (active && op != PBM_OP_ALLOC) ? a.arena[slot] : -1;
    int32_t s = 0, id = -1;
    if constexpr (K == BWalk::Collab) {
        const uint32_t gl = threadIdx.x & (uint32_t)(W - 1);
        id = walk_collab<W, Word>(a.v, need, request_seed(seed, (uint32_t)(q - gl)), lane_off,
                                  a.dedupe != 0, a.max_steps, gslots, &s);
    } else if (need) {
        const int32_t seed0 = request_seed(seed, (uint32_t)q);
        if constexpr (K == BWalk::Page) id = walk_page(a.v, seed0, a.max_steps, &s);
        else if constexpr (K == BWalk::Word32) id = walk_word<uint32_t>(a.v, seed0, a.max_steps, &s);
        else id = walk_word<uint64_t>(a.v, seed0, a.max_steps, &s);
    }
    batch_finish(a, active, op, q, slot, held, need, id, s, acc);
}

// Two requests per lane (a: q0 + lane, b: q0 + 32 + lane), one walk.
// SlotT: 32-bit arena slots when the arena has at most 2^31 of them (fewer
// instructions per request), else 64-bit.
template <typename Word, typename SlotT>
__device__ __forceinline__ void batch_round2(const BatchArgs& a, uint32_t seed, unsigned long long q0,
                                             bool act_a, int op_a, SlotT slot_a, bool act_b, int op_b,
                                             SlotT slot_b, uint32_t lane_off, BAcc& acc) {
    const bool need_a = act_a && (op_a == PBM_OP_ALLOC || op_a == PBM_OP_SWAP);
    const bool need_b = act_b && (op_b == PBM_OP_ALLOC || op_b == PBM_OP_SWAP);
    const int32_t held_a = (act_a && op_a != PBM_OP_ALLOC) ? a.arena[slot_a] : -1;
    const int32_t held_b = (act_b && op_b != PBM_OP_ALLOC) ? a.arena[slot_b] : -1;
    int32_t s = 0, id_a = -1, id_b = -1;
    walk_collab2<Word>(a.v, need_a, need_b, request_seed(seed, (uint32_t)q0), lane_off, a.dedupe != 0,
                       a.max_steps, id_a, id_b, &s);
    batch_finish(a, act_a, op_a, q0 + (threadIdx.x & 31u), slot_a, held_a, need_a, id_a, s, acc);
    batch_finish(a, act_b, op_b, q0 + 32u + (threadIdx.x & 31u), slot_b, held_b, need_b, id_b, s, acc);
}

template <typename S>
__device__ __forceinline__ S wrap_slot(S slot, S len) {
    if (slot >= len) slot = slot - len < len ? slot - len : slot % len;
    return slot;
}

// Last g in [lo, n_groups) with prefix[g] <= q (prefix[lo] <= q), searched
// by the whole warp: 32 evenly spaced probes and a ballot narrow the range
// 32-fold per round (two rounds for 256 groups).
__device__ __forceinline__ uint32_t find_group_warp(const unsigned long long* prefix, uint32_t n_groups,
                                                    unsigned long long q, uint32_t lo) {
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t hi = n_groups;
    while (hi - lo > 1u) {
        const uint32_t stride = (hi - lo + 31u) >> 5;
        const uint32_t idx = lo + lane * stride;
        const uint32_t b = __ballot_sync(0xffffffffu, idx < hi && prefix[idx] <= q);
        lo += (31u - (uint32_t)__clz((int)b)) * stride;
        hi = min(hi, lo + stride);
    }
    return lo;
}

// The persistent batch kernel.  With a.fuse each block scans the step's
// group counts into shared memory itself (no separate prefix kernel); the
// graph form's step comes with the launch's parameters (no counter to read,
// no step kernel, no grid-wide "last block" atomic at the end), so one graph
// replay is one launch.  A warp serves 32 requests (a chunk; 64 for Collab2)
// at a time.  Each block owns a contiguous range of the step's chunks and its
// warps take the next one from a shared-memory counter, so a warp whose
// chunks needed extra jumps does not hold the block's end back (static
// striding left the slowest of ~8 chunks per warp as the tail); with
// a.pools, blocks that finish their range early then drain the tail pools
// (one global counter per eighth of the grid, so no counter is hot).
// (Prefetching the next chunk's arena slots and bitmap line into L2 was
// measured slower: the extra instructions cost more than the latency they hid.)
template <BWalk K, int W, typename Word, int MINB, typename Tab, typename SlotT>
__global__ void __launch_bounds__(256, MINB) k_batch_persistent(BatchArgs a, const __grid_constant__ Tab tab) {
    extern __shared__ unsigned long long s_prefix[];
    __shared__ int32_t slots[256];
    __shared__ unsigned long long s_acc[4];
    __shared__ unsigned long long s_pool[2];   // the block's tail pool: first chunk, end
    __shared__ unsigned int s_next_chunk, s_warps_done;
    BAcc acc;
    if (threadIdx.x == 0) {
        s_next_chunk = 0u;
        s_warps_done = 0u;
    }
    if (threadIdx.x < 4u) s_acc[threadIdx.x] = 0ull;
    const uint32_t step = a.step;
    const pbm_group* groups;
    if constexpr (std::is_same<Tab, GroupTable>::value) groups = tab.g;   // read in place
    else groups = a.groups + (size_t)(step % a.n_steps) * a.n_groups;
    const uint32_t seed = a.seed + step;
    const unsigned long long* pre = a.prefix;
    if (a.fuse) {
        block_exclusive_prefix(groups, a.n_groups, s_prefix);
        pre = s_prefix;
    } else {
        __syncthreads();
    }
    if (a.pools && blockIdx.x == 0 && threadIdx.x < kPools)
        a.pools[(((step + 1u) & 1u) * kPools + threadIdx.x) * 16u] = 0ull;
    const unsigned long long total = pre[a.n_groups];
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t gl = threadIdx.x & (uint32_t)(W - 1);
    const uint32_t L = WordTraits<Word>::count(a.v);
    const uint32_t lane_off = (uint32_t)(((unsigned long long)gl * a.stride) % L);
    volatile int32_t* gslots = slots + (threadIdx.x & ~(uint32_t)(W - 1));
    constexpr unsigned long long CH = 32ull * kReqPerLane<K>;    // requests per chunk
    const unsigned long long n_chunks = (total + CH - 1ull) / CH;
    // the block's own range; with pools, the last tenth goes to the pools
    // (their bounds wait in shared memory until the range is done)
    unsigned long long per_block;
    if (a.pools) {
        per_block = (n_chunks - n_chunks / kPoolShare) / gridDim.x;
        if (threadIdx.x == 0) {
            const unsigned long long pool0 = per_block * gridDim.x;
            const unsigned long long psz = (n_chunks - pool0 + kPools - 1ull) / kPools;
            s_pool[0] = pool0 + (blockIdx.x % kPools) * psz;
            s_pool[1] = min(n_chunks, s_pool[0] + psz);
        }
        __syncthreads();
    } else {
        per_block = (n_chunks + gridDim.x - 1ull) / gridDim.x;
    }
    const unsigned long long c_begin = (unsigned long long)blockIdx.x * per_block;
    const unsigned long long c_end = min(n_chunks, c_begin + per_block);
    // the group of the warp's previous chunk: chunks only grow and a group
    // spans many chunks, so a chunk that still lies in it skips the search
    uint32_t g0 = 0;
    for (;;) {
        uint32_t k = 0;
        if (lane == 0) k = atomicAdd(&s_next_chunk, 1u);
        k = __shfl_sync(0xffffffffu, k, 0);
        unsigned long long chunk = c_begin + k;
        if (chunk >= c_end) {
            // own range done: the pool's chunks (they follow every range,
            // so the warp's chunks still only grow)
            if (!a.pools) break;
            unsigned long long j = 0;
            if (lane == 0) j = atomicAdd(a.pools + ((step & 1u) * kPools + blockIdx.x % kPools) * 16u, 1ull);
            chunk = s_pool[0] + __shfl_sync(0xffffffffu, j, 0);
            if (chunk >= s_pool[1]) break;
        }
        const unsigned long long q0 = chunk * CH;
        if (q0 >= pre[g0 + 1u]) g0 = find_group_warp(pre, a.n_groups, q0, g0);
        const unsigned long long g0_end = pre[g0 + 1u];
        // a chunk usually lies inside one group; requests past its end search on
        auto locate = [&](unsigned long long q, int& op, SlotT& slot) {
            const uint32_t g = q < g0_end ? g0 : find_group_any(pre, a.n_groups, q, g0);
            const pbm_group gd = groups[g];
            op = gd.op;
            slot = (SlotT)wrap_slot<unsigned long long>(gd.offset + (q - pre[g]), a.arena_len);
        };
        const unsigned long long q = q0 + lane;
        bool active;
        int op = PBM_OP_ALLOC;
        SlotT slot = 0;
        if constexpr (K == BWalk::Collab2) {
            const unsigned long long qb = q + 32ull;
            bool act_b;
            int op_b = PBM_OP_ALLOC;
            SlotT slot_b = 0;
            if (q0 + CH <= g0_end) {
                // the whole chunk lies in one group: its slots follow on from one base
                // (base + 63 stays below 2^32 for 32-bit slots: the arena has at most 2^31)
                const pbm_group gd = groups[g0];
                const SlotT len = (SlotT)a.arena_len;
                const SlotT base = (SlotT)wrap_slot<unsigned long long>(gd.offset + (q0 - pre[g0]), a.arena_len);
                slot = wrap_slot<SlotT>(base + (SlotT)lane, len);
                slot_b = wrap_slot<SlotT>(base + (SlotT)(32u + lane), len);
                op = gd.op;
                op_b = gd.op;
                active = true;
                act_b = true;
            } else {
                active = q < total;
                act_b = qb < total;
                if (active) locate(q, op, slot);
                if (act_b) locate(qb, op_b, slot_b);
            }
            batch_round2<Word, SlotT>(a, seed, q0, active, op, slot, act_b, op_b, slot_b, lane_off, acc);
        } else {
            active = q < total;
            if (active) locate(q, op, slot);
            batch_round<K, W, Word>(a, seed, active, op, q, (unsigned long long)slot, lane_off, gslots, acc);
        }
    }
    flush_bacc_last_warp(acc, a.stats, s_acc, &s_warps_done);
}

template <BWalk K, int W, typename Word>
__global__ void __launch_bounds__(256) k_batch_plain(BatchArgs a) {
    __shared__ int32_t slots[256];
    BAcc acc;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t gl = threadIdx.x & (uint32_t)(W - 1);
    const uint32_t L = WordTraits<Word>::count(a.v);
    const uint32_t lane_off = (uint32_t)(((unsigned long long)gl * a.stride) % L);
    volatile int32_t* gslots = slots + (threadIdx.x & ~(uint32_t)(W - 1));
    const unsigned long long warp0 = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned long long nwarps = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
    constexpr unsigned long long CH = 32ull * kReqPerLane<K>;
    for (unsigned long long chunk = warp0; chunk * CH < a.count; chunk += nwarps) {
        const unsigned long long ql = chunk * CH + lane;
        const bool active = ql < a.count;
        const unsigned long long slot = wrap_slot(a.offset + ql, a.arena_len);
        if constexpr (K == BWalk::Collab2) {
            const bool act_b = ql + 32ull < a.count;
            batch_round2<Word, unsigned long long>(a, a.seed, a.q_base + chunk * CH, active, a.op, slot, act_b, a.op,
                                                   wrap_slot(a.offset + ql + 32ull, a.arena_len), lane_off, acc);
        } else {
            batch_round<K, W, Word>(a, a.seed, active, a.op, a.q_base + ql, slot, lane_off, gslots, acc);
        }
    }
    flush_bacc(acc, a.stats);
}

}  // namespace pbm

using namespace pbm;

namespace {

// Resident blocks per SM of a persistent instantiation (queried once per block
// size, outside any stream capture).  The cache is one atomic word, (block
// size << 16) | blocks, so host threads launching batches at once never read
// a block size paired with another size's count.
template <BWalk K, int W, typename Word, int MINB, typename Tab = NoTable, typename SlotT = unsigned long long>
int persistent_blocks_per_sm(int block) {
    static std::atomic<uint32_t> cache{0u};
    const uint32_t c = cache.load(std::memory_order_relaxed);
    if ((int)(c >> 16) == block) return (int)(c & 0xffffu);
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch_persistent<K, W, Word, MINB, Tab, SlotT>, block,
                                                      kFusedPrefixBytes) != cudaSuccess) {
        cudaGetLastError();
        n = 1;
    }
    n = n > 0 ? (n < 0xffff ? n : 0xffff) : 1;
    cache.store(((uint32_t)block << 16) | (uint32_t)n, std::memory_order_relaxed);
    return n;
}

// blocks_per_sm <= 0: uncapped registers, as many blocks as fit;
// 1..kCappedBlocks-1: uncapped registers, that many blocks;
// >= kCappedBlocks: the variant whose registers are capped for kCappedBlocks
// resident blocks (5 x 256 threads: at most 51 registers, no spills for the
// collaborative walk on 32-bit words).
// grid_cap > 0: at most that many blocks (a batch whose size the host knows
// and that needs fewer blocks than fill the GPU).
template <BWalk K, int W, typename Word, typename Tab, typename SlotT>
void launch_persistent_slots(const BatchArgs& a, const Tab& tab, int block, int blocks_per_sm, size_t smem,
                             cudaStream_t s, unsigned grid_cap) {
    auto grid_of = [&](int per_sm) {
        const unsigned g = (unsigned)(sm_count() * per_sm);
        return grid_cap && grid_cap < g ? grid_cap : g;
    };
    if (blocks_per_sm >= kCappedBlocks) {
        int fit = persistent_blocks_per_sm<K, W, Word, kCappedBlocks, Tab, SlotT>(block);
        int per_sm = blocks_per_sm < fit ? blocks_per_sm : fit;
        k_batch_persistent<K, W, Word, kCappedBlocks, Tab, SlotT><<<grid_of(per_sm), block, smem, s>>>(a, tab);
    } else {
        int fit = persistent_blocks_per_sm<K, W, Word, 1, Tab, SlotT>(block);
        int per_sm = (blocks_per_sm > 0 && blocks_per_sm < fit) ? blocks_per_sm : fit;
        k_batch_persistent<K, W, Word, 1, Tab, SlotT><<<grid_of(per_sm), block, smem, s>>>(a, tab);
    }
}

// 32-bit arena slots for the two-requests-per-lane walk when the arena has at
// most 2^31 slots; every other walk keeps 64-bit slots.
constexpr unsigned long long kSlot32Max = 1ull << 31;

template <BWalk K> constexpr bool kHasSlot32 = K == BWalk::Collab2;

template <BWalk K, int W, typename Word, typename Tab>
void launch_persistent(const BatchArgs& a, const Tab& tab, int block, int blocks_per_sm, size_t smem,
                       cudaStream_t s, unsigned grid_cap) {
    if constexpr (kHasSlot32<K>) {
        if (a.arena_len <= kSlot32Max) {
            launch_persistent_slots<K, W, Word, Tab, uint32_t>(a, tab, block, blocks_per_sm, smem, s, grid_cap);
            return;
        }
    }
    launch_persistent_slots<K, W, Word, Tab, unsigned long long>(a, tab, block, blocks_per_sm, smem, s, grid_cap);
}

// tab: the inline descriptor table of a launch-form batch (null: a.groups).
template <BWalk K, int W, typename Word>
int launch_batch_kw(const BatchArgs& a, bool persistent, int block, int blocks_per_sm, cudaStream_t s,
                    const GroupTable* tab, unsigned grid_cap) {
    if (persistent) {
        const size_t smem = a.fuse ? sizeof(unsigned long long) * (a.n_groups + 1u) : 0u;
        if (tab) launch_persistent<K, W, Word>(a, *tab, block, blocks_per_sm, smem, s, grid_cap);
        else launch_persistent<K, W, Word>(a, NoTable{}, block, blocks_per_sm, smem, s, grid_cap);
    } else {
        const unsigned long long per_warp = 32ull * kReqPerLane<K>;
        unsigned long long warps = (a.count + per_warp - 1ull) / per_warp;
        unsigned long long grid = (warps * 32ull + (unsigned long long)block - 1ull) / (unsigned long long)block;
        if (grid < 1) grid = 1;
        k_batch_plain<K, W, Word><<<(unsigned)grid, block, 0, s>>>(a);
    }
    PBM_LAUNCH_CHECK();
    return PBM_OK;
}

int launch_batch(const pbm_walk_config* c, const BatchArgs& a, bool persistent, cudaStream_t s,
                 const GroupTable* tab = nullptr, unsigned grid_cap = 0) {
    const int block = c->block_size ? c->block_size : kDefaultBlock;
    const int bps = c->blocks_per_sm;
    const bool w64 = c->word_bits == 64;
    switch (c->strategy) {
    case PBM_RANDOM_WALK:
        return launch_batch_kw<BWalk::Page, 32, uint32_t>(a, persistent, block, bps, s, tab, grid_cap);
    case PBM_RANDOM_WALK_BM:
        return w64 ? launch_batch_kw<BWalk::Word64, 32, uint64_t>(a, persistent, block, bps, s, tab, grid_cap)
                   : launch_batch_kw<BWalk::Word32, 32, uint32_t>(a, persistent, block, bps, s, tab, grid_cap);
    case PBM_COLLAB_RW_BM: {
        const int W = c->collab_width ? c->collab_width : 32;
        if (W == 64) return w64 ? launch_batch_kw<BWalk::Collab2, 32, uint64_t>(a, persistent, block, bps, s, tab, grid_cap)
                                : launch_batch_kw<BWalk::Collab2, 32, uint32_t>(a, persistent, block, bps, s, tab, grid_cap);
        if (W == 8) return w64 ? launch_batch_kw<BWalk::Collab, 8, uint64_t>(a, persistent, block, bps, s, tab, grid_cap)
                               : launch_batch_kw<BWalk::Collab, 8, uint32_t>(a, persistent, block, bps, s, tab, grid_cap);
        if (W == 16) return w64 ? launch_batch_kw<BWalk::Collab, 16, uint64_t>(a, persistent, block, bps, s, tab, grid_cap)
                                : launch_batch_kw<BWalk::Collab, 16, uint32_t>(a, persistent, block, bps, s, tab, grid_cap);
        return w64 ? launch_batch_kw<BWalk::Collab, 32, uint64_t>(a, persistent, block, bps, s, tab, grid_cap)
                   : launch_batch_kw<BWalk::Collab, 32, uint32_t>(a, persistent, block, bps, s, tab, grid_cap);
    }
    default:
        return PBM_ERR_UNSUPPORTED;
    }
}

// Blocks per SM the persistent launch of this configuration will use
// (resolved before a capture, so the capture issues no occupancy query).
int resolve_blocks_per_sm(const pbm_walk_config* c, unsigned long long arena_len) {
    const int block = c->block_size ? c->block_size : kDefaultBlock;
    const bool slot32 = arena_len <= kSlot32Max;
    const bool w64 = c->word_bits == 64;
    const bool capped = c->blocks_per_sm >= kCappedBlocks;
    auto pick = [&](int fit1, int fitc) {
        if (capped) return c->blocks_per_sm < fitc ? c->blocks_per_sm : fitc;
        return (c->blocks_per_sm > 0 && c->blocks_per_sm < fit1) ? c->blocks_per_sm : fit1;
    };
#define PBM_FITS(K, W, T) \
    pick(persistent_blocks_per_sm<K, W, T, 1>(block), persistent_blocks_per_sm<K, W, T, kCappedBlocks>(block))
    switch (c->strategy) {
    case PBM_RANDOM_WALK: return PBM_FITS(BWalk::Page, 32, uint32_t);
    case PBM_RANDOM_WALK_BM:
        return w64 ? PBM_FITS(BWalk::Word64, 32, uint64_t) : PBM_FITS(BWalk::Word32, 32, uint32_t);
    default: {
        const int W = c->collab_width ? c->collab_width : 32;
        if (W == 64 && slot32)
            return w64 ? pick(persistent_blocks_per_sm<BWalk::Collab2, 32, uint64_t, 1, NoTable, uint32_t>(block),
                              persistent_blocks_per_sm<BWalk::Collab2, 32, uint64_t, kCappedBlocks, NoTable, uint32_t>(block))
                       : pick(persistent_blocks_per_sm<BWalk::Collab2, 32, uint32_t, 1, NoTable, uint32_t>(block),
                              persistent_blocks_per_sm<BWalk::Collab2, 32, uint32_t, kCappedBlocks, NoTable, uint32_t>(block));
        if (W == 64) return w64 ? PBM_FITS(BWalk::Collab2, 32, uint64_t) : PBM_FITS(BWalk::Collab2, 32, uint32_t);
        if (W == 8) return w64 ? PBM_FITS(BWalk::Collab, 8, uint64_t) : PBM_FITS(BWalk::Collab, 8, uint32_t);
        if (W == 16) return w64 ? PBM_FITS(BWalk::Collab, 16, uint64_t) : PBM_FITS(BWalk::Collab, 16, uint32_t);
        return w64 ? PBM_FITS(BWalk::Collab, 32, uint64_t) : PBM_FITS(BWalk::Collab, 32, uint32_t);
    }
    }
#undef PBM_FITS
}

BatchArgs base_args(pbm_pool* p, const pbm_walk_config* c, int32_t* arena, uint64_t arena_len,
                    uint32_t seed, int32_t* d_steps) {
    BatchArgs a{};
    a.v = p->view;
    a.seed = seed;
    a.arena = arena;
    a.arena_len = arena_len;
    a.steps = d_steps;
    a.max_steps = c->max_steps ? c->max_steps : kDefaultMaxSteps;
    a.stride = c->stride ? c->stride : 1u;
    a.merge = c->free_merge;
    a.stats = p->d_stats;
    a.n_steps = 1u;
    const int Wc = c->strategy == PBM_COLLAB_RW_BM ? (c->collab_width ? c->collab_width : 32) : 1;
    const int W = Wc == 64 ? 32 : Wc;   // lanes reading the window
    const uint32_t L = c->word_bits == 64 ? p->view.n_words64 : p->view.n_words32;
    a.dedupe = ((unsigned long long)(W - 1) * a.stride >= L) ? 1 : 0;
    return a;
}

int valid_cfg(const pbm_walk_config* c) {
    if (!c) return PBM_ERR_INVALID;
    if (c->word_bits != 0 && c->word_bits != 32 && c->word_bits != 64) return PBM_ERR_INVALID;
    if (c->collab_width != 0 && c->collab_width != 8 && c->collab_width != 16 && c->collab_width != 32 &&
        !(c->collab_width == 64 && c->strategy == PBM_COLLAB_RW_BM))
        return PBM_ERR_INVALID;
    if (c->block_size < 0 || c->block_size > 256 || (c->block_size % 32) != 0) return PBM_ERR_INVALID;
    if (c->strategy != PBM_RANDOM_WALK && c->strategy != PBM_RANDOM_WALK_BM && c->strategy != PBM_COLLAB_RW_BM)
        return PBM_ERR_UNSUPPORTED;
    return PBM_OK;
}

}  // namespace

extern "C" {

int pbm_batch_launch_results(pbm_pool* pool, const pbm_walk_config* cfg, const pbm_group* d_groups,
                             const pbm_group* h_groups, uint32_t n_groups, int32_t* d_arena, uint64_t arena_len,
                             uint32_t seed, int32_t* d_steps, int32_t* results, int mode, void* stream) {
    PBM_ON_POOL_DEVICE(pool);
    if (!pool || !d_arena || arena_len == 0) return PBM_ERR_INVALID;
    int rc = valid_cfg(cfg);
    if (rc) return rc;
    if (results && !device_writable(results)) return PBM_ERR_INVALID;
    if (n_groups == 0) return PBM_OK;
    cudaStream_t s = (cudaStream_t)stream;
    pool->fifo_valid = false;
    BatchArgs a = base_args(pool, cfg, d_arena, arena_len, seed, d_steps);
    a.results = results;
    if (mode == PBM_LAUNCH_PLAIN) {
        if (!h_groups) return PBM_ERR_INVALID;
        unsigned long long q = 0;
        for (uint32_t g = 0; g < n_groups; ++g) {
            const pbm_group& gd = h_groups[g];
            if (gd.op < PBM_OP_ALLOC || gd.op > PBM_OP_SWAP) return PBM_ERR_INVALID;
            if (gd.count == 0) continue;
            a.op = gd.op;
            a.count = gd.count;
            a.offset = gd.offset;
            a.q_base = q;
            rc = launch_batch(cfg, a, false, s);
            if (rc) return rc;
            q += gd.count;
        }
        return PBM_OK;
    }
    if (mode != PBM_LAUNCH_PERSISTENT) return PBM_ERR_INVALID;
    if (!d_groups) {                   // host table carried in the launch's parameters
        if (!h_groups || n_groups > PBM_MAX_INLINE_GROUPS) return PBM_ERR_INVALID;
        GroupTable tab{};
        unsigned long long total = 0;
        for (uint32_t g = 0; g < n_groups; ++g) {
            if (h_groups[g].op < PBM_OP_ALLOC || h_groups[g].op > PBM_OP_SWAP) return PBM_ERR_INVALID;
            tab.g[g] = h_groups[g];
            total += h_groups[g].count;
        }
        if (total == 0) return PBM_OK;
        a.n_groups = n_groups;
        a.fuse = 1;
        // the host knows the batch's size: no more blocks than chunks for one
        // chunk per warp (a small batch launches one block, not a full grid)
        const unsigned long long per_chunk = (cfg->strategy == PBM_COLLAB_RW_BM && cfg->collab_width == 64) ? 64ull : 32ull;
        const unsigned long long warps = (unsigned long long)(cfg->block_size ? cfg->block_size : kDefaultBlock) / 32ull;
        const unsigned long long need = ((total + per_chunk - 1ull) / per_chunk + warps - 1ull) / warps;
        return launch_batch(cfg, a, true, s, &tab, (unsigned)(need < 0xffffffffull ? need : 0xffffffffull));
    }
    a.groups = d_groups;
    a.n_groups = n_groups;
    if (n_groups <= kFusedGroups) {   // every block scans the groups itself
        a.fuse = 1;
        return launch_batch(cfg, a, true, s);
    }
    if (pool->prefix_cap < n_groups + 1u) {
        cudaFree(pool->d_prefix);
        pool->d_prefix = nullptr;
        if (cudaMalloc(&pool->d_prefix, sizeof(unsigned long long) * (n_groups + 1u)) != cudaSuccess) {
            cudaGetLastError();
            pool->prefix_cap = 0;
            return PBM_ERR_NOMEM;
        }
        pool->prefix_cap = n_groups + 1u;
    }
    k_batch_prefix<<<1, 1024, 0, s>>>(d_groups, n_groups, nullptr, 0u, 1u, pool->d_prefix);
    PBM_LAUNCH_CHECK();
    a.groups = d_groups;
    a.n_groups = n_groups;
    a.prefix = pool->d_prefix;
    return launch_batch(cfg, a, true, s);
}

int pbm_batch_launch(pbm_pool* pool, const pbm_walk_config* cfg, const pbm_group* d_groups,
                     const pbm_group* h_groups, uint32_t n_groups, int32_t* d_arena,
                     uint64_t arena_len, uint32_t seed, int32_t* d_steps, int mode, void* stream) {
    PBM_ON_POOL_DEVICE(pool);
    return pbm_batch_launch_results(pool, cfg, d_groups, h_groups, n_groups, d_arena, arena_len, seed, d_steps,
                                    nullptr, mode, stream);
}

int pbm_batch_graph_create(pbm_pool* pool, const pbm_walk_config* cfg, const pbm_group* d_groups,
                           uint32_t n_groups, uint32_t n_steps, int32_t* d_arena, uint64_t arena_len,
                           uint32_t seed0, void* stream, pbm_graph** out) {
    PBM_ON_POOL_DEVICE(pool);
    return pbm_batch_graph_create_results(pool, cfg, d_groups, n_groups, n_steps, d_arena, arena_len, seed0, nullptr,
                                          stream, out);
}

int pbm_batch_graph_create_results(pbm_pool* pool, const pbm_walk_config* cfg, const pbm_group* d_groups,
                                   uint32_t n_groups, uint32_t n_steps, int32_t* d_arena, uint64_t arena_len,
                                   uint32_t seed0, int32_t* results, void* stream, pbm_graph** out) {
    PBM_ON_POOL_DEVICE(pool);
    if (!pool || !d_groups || !d_arena || !out || n_groups == 0 || n_steps == 0 || arena_len == 0)
        return PBM_ERR_INVALID;
    if (results && !device_writable(results)) return PBM_ERR_INVALID;
    int rc = valid_cfg(cfg);
    if (rc) return rc;
    *out = nullptr;
    cudaStream_t s = (cudaStream_t)stream;
    pbm_graph* g = new (std::nothrow) pbm_graph();   // value-initialised: null handles, step 0
    if (!g) return PBM_ERR_NOMEM;
    g->device = pool->device;
    const size_t pool_bytes = sizeof(unsigned long long) * 2u * kPools * 16u;
    if (cudaMalloc(&g->d_pools, pool_bytes) != cudaSuccess ||
        cudaMalloc(&g->d_prefix, sizeof(unsigned long long) * (n_groups + 1u)) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(g->d_pools);
        delete g;
        return PBM_ERR_NOMEM;
    }
    auto fail = [&](int code) {
        if (g->exec) cudaGraphExecDestroy(g->exec);
        if (g->graph) cudaGraphDestroy(g->graph);
        cudaFree(g->d_pools);
        cudaFree(g->d_prefix);
        delete g;
        cudaGetLastError();
        return code;
    };
    if (cudaMemsetAsync(g->d_pools, 0, pool_bytes, s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess)
        return fail(PBM_ERR_CUDA);
    BatchArgs a = base_args(pool, cfg, d_arena, arena_len, seed0, nullptr);
    a.results = results;
    a.groups = d_groups;
    a.n_groups = n_groups;
    a.prefix = g->d_prefix;
    a.step = 0u;                              // written before each replay
    a.n_steps = n_steps;
    a.pools = g->d_pools;
    a.fuse = n_groups <= kFusedGroups ? 1 : 0;
    static_assert(sizeof(BatchArgs) <= sizeof(g->batch_args), "graph keeps the kernel's arguments");
    std::memcpy(g->batch_args, &a, sizeof(a));
    g->prefix_groups = d_groups;
    g->prefix_n_groups = n_groups;
    g->prefix_n_steps = n_steps;
    g->prefix_out = g->d_prefix;
    // Capture on a private stream (the legacy default stream cannot be
    // captured); the graph is replayed later on the caller's stream.  The
    // occupancy query runs before capture.
    pbm_walk_config c2 = *cfg;
    resolve_blocks_per_sm(cfg, arena_len);   // fills the occupancy caches before the capture starts
    cudaStream_t cap = nullptr;
    if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess) return fail(PBM_ERR_CUDA);
    const unsigned long long before = g_launches.load();
    cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        cudaStreamDestroy(cap);
        return fail(PBM_ERR_CUDA);
    }
    if (!a.fuse) {
        k_batch_prefix<<<1, 1024, 0, cap>>>(d_groups, n_groups, nullptr, 0u, n_steps, g->d_prefix);
        count_launch();
    }
    rc = launch_batch(&c2, a, true, cap);
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(cap, &graph);
    cudaStreamDestroy(cap);
    g->graph = graph;
    if (rc || e != cudaSuccess) return fail(rc ? rc : PBM_ERR_CUDA);
    // the kernel nodes whose parameters carry the step
    size_t nn = 0;
    if (cudaGraphGetNodes(graph, nullptr, &nn) != cudaSuccess) return fail(PBM_ERR_CUDA);
    std::vector<cudaGraphNode_t> nodes(nn);
    if (nn && cudaGraphGetNodes(graph, nodes.data(), &nn) != cudaSuccess) return fail(PBM_ERR_CUDA);
    for (cudaGraphNode_t node : nodes) {
        cudaGraphNodeType t;
        cudaKernelNodeParams kp{};
        if (cudaGraphNodeGetType(node, &t) != cudaSuccess || t != cudaGraphNodeTypeKernel) continue;
        if (cudaGraphKernelNodeGetParams(node, &kp) != cudaSuccess) return fail(PBM_ERR_CUDA);
        kp.kernelParams = nullptr;   // pointed into the graph; replays pass their own
        kp.extra = nullptr;
        if (kp.func == (void*)k_batch_prefix) {
            g->prefix_node = node;
            g->prefix_kp = kp;
        } else {
            g->batch_node = node;
            g->batch_kp = kp;
        }
    }
    if (!g->batch_node || (!a.fuse && !g->prefix_node)) return fail(PBM_ERR_CUDA);
    if (cudaGraphInstantiate(&g->exec, graph, 0) != cudaSuccess) return fail(PBM_ERR_CUDA);
    g->launches_per_replay = g_launches.load() - before;
    // capture does not launch: take the counted launches back
    g_launches.fetch_sub(g->launches_per_replay);
    pool->fifo_valid = false;
    *out = g;
    return PBM_OK;
}

int pbm_graph_replay(pbm_graph* g, void* stream) {
    if (!g || !g->exec) return PBM_ERR_INVALID;
    pbm::DeviceScope scope(g->device);
    if (g->batch_node) {
        // this replay's step goes into the kernels' parameters (a host-side
        // update of the instantiated graph; launches already queued keep theirs)
        BatchArgs a;
        std::memcpy(&a, g->batch_args, sizeof(a));
        a.step = g->host_step;
        NoTable tab{};
        void* args[2] = {&a, &tab};
        cudaKernelNodeParams kp = g->batch_kp;
        kp.kernelParams = args;
        PBM_CUDA_TRY(cudaGraphExecKernelNodeSetParams(g->exec, g->batch_node, &kp));
        if (g->prefix_node) {
            const pbm_group* groups = g->prefix_groups;
            uint32_t n_groups = g->prefix_n_groups, step = g->host_step, n_steps = g->prefix_n_steps;
            const uint32_t* no_counter = nullptr;
            unsigned long long* prefix = g->prefix_out;
            void* pargs[6] = {&groups, &n_groups, &no_counter, &step, &n_steps, &prefix};
            cudaKernelNodeParams pkp = g->prefix_kp;
            pkp.kernelParams = pargs;
            PBM_CUDA_TRY(cudaGraphExecKernelNodeSetParams(g->exec, g->prefix_node, &pkp));
        }
        ++g->host_step;
    }
    PBM_CUDA_TRY(cudaGraphLaunch(g->exec, (cudaStream_t)stream));
    count_launch(g->launches_per_replay);
    return PBM_OK;
}

int pbm_graph_set_step(pbm_graph* g, uint32_t step, void* stream) {
    if (!g) return PBM_ERR_INVALID;
    pbm::DeviceScope scope(g->device);
    cudaStream_t s = (cudaStream_t)stream;
    if (g->batch_node) {
        g->host_step = step;
        // both parities of the tail pools start empty again
        PBM_CUDA_TRY(cudaMemsetAsync(g->d_pools, 0, sizeof(unsigned long long) * 2u * kPools * 16u, s));
    } else {
        PBM_CUDA_TRY(cudaMemcpyAsync(g->d_step, &step, sizeof(step), cudaMemcpyHostToDevice, s));
    }
    PBM_CUDA_TRY(cudaStreamSynchronize(s));
    return PBM_OK;
}

int pbm_graph_destroy(pbm_graph* g) {
    if (!g) return PBM_ERR_INVALID;
    pbm::DeviceScope scope(g->device);
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    cudaFree(g->d_step);
    cudaFree(g->d_pools);
    cudaFree(g->d_prefix);
    delete g;
    return PBM_OK;
}

}  // extern "C"
