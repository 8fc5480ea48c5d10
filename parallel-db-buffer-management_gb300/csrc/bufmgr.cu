// bufmgr.cu -- buffer manager with CLOCK (second-chance) replacement.
//
// The reference has page allocators only; its SingleClock / DistClock arms
// sweep the free map (parallelPage.cu:491-509, 571-592) but there is no page
// table, no reference bits and no eviction.  This file defines the buffer
// manager on those sweep mechanics:
//
//   page_table[p]   frame holding logical page p, -1 not resident, -2 being
//                   loaded by another request
//   frame_state[f]  (page << 32) | pins in one 64-bit word.  A fetch pins with
//                   one atomicAdd and keeps the pin only if the word it added
//                   to still named its page (else it subtracts it again), so
//                   hot frames see no compare-and-swap retries; a sweep takes
//                   a frame only if it is unpinned and unchanged (one CAS), so
//                   a pin in flight makes the sweep pass the frame by
//   ref[f]          CLOCK reference bit, set on every fetch
//   arms            SINGLE: one shared hand (atomicAdd); DIST: per-slot hands,
//                   each starting at its own frame and advancing privately
//
// fetch(p): resident -> pin it, set ref (hit).  Not resident -> become its
// loader (CAS page_table -1 -> -2), sweep: skip pinned frames, clear the
// reference bit of referenced ones (second chance), take the first unpinned
// unreferenced frame, unmap its old page (eviction), optionally copy the
// page from the backing store, map p (miss).  A fetch that finds no frame
// within max_sweep hand steps fails (-1) instead of spinning; waits on a
// loading page are bounded too.  Lanes of a warp that fetch the same page
// pin it with one atomicAdd of their count (Zipf streams repeat hot pages
// within a warp).
#include <cstring>
#include <new>

#include "internal.cuh"

namespace pbm {
namespace {

constexpr uint32_t kEmptyPage = 0xffffffffu;
constexpr int32_t kLoading = -2;
constexpr uint32_t kFetchSpinLimit = 1u << 16;

struct BmStats {
    unsigned long long hits, misses, evictions, failures, unpins, bad_unpins, timeouts, pad;
};

struct BmView {
    int32_t* page_table;
    unsigned long long* frame_state;
    uint8_t* ref;
    unsigned long long* single_hand;
    uint32_t* arms;
    const char* backing;     // n_logical * frame_size bytes, may be null
    char* frames;            // n_frames * frame_size bytes, may be null
    BmStats* stats;
    uint32_t n_logical;
    uint32_t n_frames;
    uint32_t frame_size;
    uint32_t max_sweep;
    uint32_t n_arms;
    int32_t dist;            // 0 = single hand, 1 = per-slot hands
};

// Shared-hand positions a sweeping thread takes per atomic in parallel rounds.
// Measured on the Zipf(0.99) trace: 8 raised fetches/s by 20% but dropped the
// hit rate from 85.2% to 82.1% (positions reserved past the victim are
// skipped, so the hand laps faster than frames are examined) and slowed the
// 4 KiB-copy form by 37%; 2 kept the hit rate and gained nothing.  So the
// hand moves one position per atomic, as the reference's SingleClock arm.
constexpr uint32_t kHandBatch = 1;

// Per-slot hand (DistClock, parallelPage.cu:571-592): the slot's hand is
// private, so it reads the next kLookahead frames' words and reference bits
// in one round trip and then examines them in hand order exactly as the
// one-step sweep does, stopping at the victim (the hand ends just past it,
// and frames beyond it are untouched).  Never more frames at once than the
// pool has, so one batch never sees a frame twice.
constexpr uint32_t kLookahead = 8;

__device__ __forceinline__ int32_t sweep_private(const BmView& b, uint32_t page, uint32_t slot,
                                                 uint32_t* old_page) {
    uint32_t arm = b.arms[slot];
    if (arm >= b.n_frames) arm %= b.n_frames;
    const uint32_t width = b.n_frames < kLookahead ? b.n_frames : kLookahead;
    int32_t out = -1;
    for (uint32_t done = 0; done < b.max_sweep && out < 0;) {
        unsigned long long st[kLookahead];
        uint8_t rf[kLookahead];
#pragma unroll
        for (uint32_t j = 0; j < kLookahead; ++j) {
            if (j < width) {
                uint32_t f = arm + j;
                if (f >= b.n_frames) f -= b.n_frames;
                st[j] = __ldcg(b.frame_state + f);
                rf[j] = b.ref[f];
            }
        }
#pragma unroll
        for (uint32_t j = 0; j < kLookahead; ++j) {
            if (j >= width || done >= b.max_sweep || out >= 0) break;
            const uint32_t f = arm;
            arm = f + 1u == b.n_frames ? 0u : f + 1u;
            ++done;
            if ((uint32_t)st[j] != 0u) continue;                // pinned
            if (rf[j]) { b.ref[f] = 0; continue; }              // second chance
            const unsigned long long ns = ((unsigned long long)page << 32) | 1ull;
            if (atomicCAS(b.frame_state + f, st[j], ns) == st[j]) {
                *old_page = (uint32_t)(st[j] >> 32);
                out = (int32_t)f;
            }
        }
    }
    b.arms[slot] = arm;
    return out;
}

// Victim search; returns a frame now holding (page, 1 pin) and its old page.
// The shared hand advances `batch` positions per atomic, which the sweeping
// thread then examines in order (parallelPage.cu:491-509 steps it by one).
template <bool DIST>
__device__ __forceinline__ int32_t sweep(const BmView& b, uint32_t page, uint32_t slot, uint32_t batch,
                                         uint32_t* old_page) {
    if constexpr (DIST) return sweep_private(b, page, slot, old_page);
    unsigned long long res = 0;
    uint32_t res_left = 0;
    int32_t out = -1;
    for (uint32_t i = 0; i < b.max_sweep; ++i) {
        if (res_left == 0u) {
            res = atomicAdd(b.single_hand, (unsigned long long)batch);
            res_left = batch;
        }
        const uint32_t f = (uint32_t)((res + (batch - res_left)) % b.n_frames);
        --res_left;
        unsigned long long s = __ldcg(b.frame_state + f);
        if ((uint32_t)s != 0u) continue;                    // pinned
        if (b.ref[f]) { b.ref[f] = 0; continue; }           // second chance
        unsigned long long ns = ((unsigned long long)page << 32) | 1ull;
        if (atomicCAS(b.frame_state + f, s, ns) == s) {
            *old_page = (uint32_t)(s >> 32);
            out = (int32_t)f;
            break;
        }
    }
    return out;
}

struct BmAcc {
    unsigned long long hits = 0, misses = 0, evictions = 0, failures = 0, timeouts = 0;
};

// Adds k pins to frame f if it holds `page`; otherwise leaves it unchanged
// (the add is taken back) and returns false.
__device__ __forceinline__ bool pin_if_owner(const BmView& b, int32_t f, uint32_t page, uint32_t k) {
    const unsigned long long old = atomicAdd(b.frame_state + f, (unsigned long long)k);
    if ((uint32_t)(old >> 32) == page) return true;
    atomicAdd(b.frame_state + f, 0ull - (unsigned long long)k);
    return false;
}

template <bool DIST>
__device__ __forceinline__ int32_t fetch(const BmView& b, uint32_t page, uint32_t slot, uint32_t batch, BmAcc& acc) {
    for (uint32_t attempt = 0; attempt < kFetchSpinLimit; ++attempt) {
        int32_t f = __ldcg(b.page_table + page);
        if (f >= 0) {
            if (pin_if_owner(b, f, page, 1u)) {
                b.ref[f] = 1;
                ++acc.hits;
                return f;
            }
            continue;   // the frame changed owner: read the page table again
        }
        if (f == -1) {
            if (atomicCAS(b.page_table + page, -1, kLoading) != -1) continue;
            uint32_t old_page = kEmptyPage;
            int32_t h = sweep<DIST>(b, page, slot, batch, &old_page);
            if (h < 0) {
                atomicExch(b.page_table + page, -1);
                ++acc.failures;
                return -1;
            }
            if (old_page != kEmptyPage) {
                atomicExch(b.page_table + old_page, -1);
                ++acc.evictions;
            }
            if (b.backing && b.frames) {
                const int4* src = reinterpret_cast<const int4*>(b.backing + (size_t)page * b.frame_size);
                int4* dst = reinterpret_cast<int4*>(b.frames + (size_t)h * b.frame_size);
                for (uint32_t k = 0; k < b.frame_size / 16u; ++k) dst[k] = src[k];
            }
            b.ref[h] = 1;
            __threadfence();
            atomicExch(b.page_table + page, h);
            ++acc.misses;
            return h;
        }
        __nanosleep(32);   // another request is loading this page
    }
    ++acc.timeouts;
    return -1;
}

// Warp-cooperative CLOCK sweep on the single hand.  The lanes in `loaders`
// (each the loader of its own `page`, its page-table entry already set to
// loading) need victim frames.  Per batch the warp takes 32 consecutive hand
// positions with one atomicAdd and every lane examines one frame, as the
// one-thread sweep does: a pinned frame is passed, a referenced one loses its
// reference bit (second chance), an unpinned unreferenced one is a candidate.
// Candidates go in hand order to the loaders in lane order, each taken with
// the one-thread sweep's CAS (a pin that arrived in between makes it fail and
// the loader waits for the next batch); candidates beyond the loaders' need
// are passed.  A loader gives up after its max_sweep positions.  So a miss
// costs about one batch of round trips instead of one per frame examined.
// The whole warp calls converged; returns the lane's frame (-1 if none) and
// the page it held.
__device__ __forceinline__ int32_t sweep_warp(const BmView& b, uint32_t loaders, uint32_t page,
                                              uint32_t* old_page) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t lt = (1u << lane) - 1u;
    int32_t out = -1;
    const uint32_t max_batches = b.max_sweep > 32u ? (b.max_sweep + 31u) / 32u : 1u;
    for (uint32_t it = 0; loaders != 0u && it < max_batches; ++it) {
        unsigned long long base = 0;
        if (lane == 0u) base = atomicAdd(b.single_hand, 32ull);
        base = __shfl_sync(0xffffffffu, base, 0);
        const uint32_t f = (uint32_t)((base + lane) % b.n_frames);
        const unsigned long long st = __ldcg(b.frame_state + f);
        bool cand = false;
        if ((uint32_t)st == 0u) {                   // unpinned
            if (b.ref[f]) b.ref[f] = 0;             // second chance
            else cand = true;
        }
        const uint32_t cm = __ballot_sync(0xffffffffu, cand);
        const int n_load = __popc(loaders);
        // candidate of rank k serves the loader of rank k
        const int k = __popc(cm & lt);
        const int target = (cand && k < n_load) ? (int)nth_set_bit(loaders, k) : -1;
        const uint32_t tpage = __shfl_sync(0xffffffffu, page, target < 0 ? (int)lane : target);
        bool took = false;
        if (target >= 0) {
            const unsigned long long ns = ((unsigned long long)tpage << 32) | 1ull;
            took = atomicCAS(b.frame_state + f, st, ns) == st;
        }
        const uint32_t tm = __ballot_sync(0xffffffffu, took);
        const bool is_loader = (loaders >> lane) & 1u;
        const int r = __popc(loaders & lt);
        const int src = (is_loader && r < __popc(cm)) ? (int)nth_set_bit(cm, r) : -1;
        const uint32_t got_f = __shfl_sync(0xffffffffu, f, src < 0 ? (int)lane : src);
        const unsigned long long got_s = __shfl_sync(0xffffffffu, st, src < 0 ? (int)lane : src);
        if (src >= 0 && ((tm >> src) & 1u)) {
            out = (int32_t)got_f;
            *old_page = (uint32_t)(got_s >> 32);
        }
        loaders = __ballot_sync(0xffffffffu, is_loader && out < 0);
    }
    return out;
}

// The loaders' side of a cooperative miss: unmap the victims' old pages, copy
// each new page from the backing store with the whole warp (one loader at a
// time, 16 bytes per lane per step), then publish the page-table entries.
// The whole warp calls converged; h = the lane's frame from sweep_warp.
__device__ __forceinline__ void finish_loads_warp(const BmView& b, bool loader, uint32_t page, int32_t h,
                                                  uint32_t old_page, BmAcc& acc) {
    if (loader) {
        if (h < 0) {
            atomicExch(b.page_table + page, -1);
            ++acc.failures;
        } else if (old_page != kEmptyPage) {
            atomicExch(b.page_table + old_page, -1);
            ++acc.evictions;
        }
    }
    if (b.backing && b.frames) {
        const uint32_t lane = threadIdx.x & 31u;
        const uint32_t n16 = b.frame_size / 16u;
        uint32_t todo = __ballot_sync(0xffffffffu, loader && h >= 0);
        while (todo) {
            const int l = __ffs((int)todo) - 1;
            todo &= todo - 1u;
            const uint32_t pg = __shfl_sync(0xffffffffu, page, l);
            const int32_t fr = __shfl_sync(0xffffffffu, h, l);
            const int4* src = reinterpret_cast<const int4*>(b.backing + (size_t)pg * b.frame_size);
            int4* dst = reinterpret_cast<int4*>(b.frames + (size_t)fr * b.frame_size);
            for (uint32_t k = lane; k < n16; k += 32u) dst[k] = src[k];
        }
        __threadfence();
        __syncwarp();
    }
    if (loader && h >= 0) {
        b.ref[h] = 1;
        __threadfence();
        atomicExch(b.page_table + page, h);
        ++acc.misses;
    }
}

// Releases k pins of frame f with one atomic.  A release of more pins than
// the frame holds (a caller error) is taken back and counted as bad; its
// subtraction can borrow from the page field for that instant, which makes a
// racing fetch see another page and retry, and a racing sweep's CAS fail.
__device__ __forceinline__ void unpin_k(const BmView& b, int32_t f, uint32_t k, unsigned long long& ok,
                                        unsigned long long& bad) {
    if (f < 0 || (uint32_t)f >= b.n_frames || k == 0u) return;
    const unsigned long long old = atomicAdd(b.frame_state + f, 0ull - (unsigned long long)k);
    if ((uint32_t)old < k) {
        atomicAdd(b.frame_state + f, (unsigned long long)k);
        bad += k;
        return;
    }
    ok += k;
}

// One round: release the listed pins, then fetch this round's pages.
// With one thread this is the deterministic replay of the round.
// DIST: per-slot hands (b.dist), else the single shared hand.
template <bool DIST>
__global__ void __launch_bounds__(256) k_round(BmView b, const int32_t* release_frames_of,
                                               const int32_t* release_idx, uint32_t n_release,
                                               const int32_t* pages, uint32_t n, uint32_t slot0,
                                               int32_t* frames_out) {
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t nthr = (uint64_t)gridDim.x * blockDim.x;
    unsigned long long ok = 0, bad = 0;
    if (nthr == 1u) {
        for (uint32_t j = 0; j < n_release; ++j) unpin_k(b, release_frames_of[release_idx[j]], 1u, ok, bad);
    } else {
        // warp-uniform trip count: lanes releasing pins of the same frame (hot
        // pages of a skewed stream) merge them into one atomic
        const uint32_t lane = threadIdx.x & 31u;
        for (uint64_t base = tid - lane; base < n_release; base += nthr) {
            const uint64_t j = base + lane;
            const int32_t f = j < n_release ? release_frames_of[release_idx[j]] : -1;
            const bool valid = f >= 0 && (uint32_t)f < b.n_frames;
            const uint32_t peers = __match_any_sync(0xffffffffu, valid ? (uint32_t)f : 0x80000000u + lane);
            if (valid && (uint32_t)(__ffs((int)peers) - 1) == lane) unpin_k(b, f, (uint32_t)__popc(peers), ok, bad);
        }
    }
    BmAcc acc;
    if (nthr == 1u) {
        __threadfence();
        for (uint32_t i = 0; i < n; ++i) {
            int32_t p = pages[i];
            int32_t f = -1;
            if (p >= 0 && (uint32_t)p < b.n_logical) f = fetch<DIST>(b, (uint32_t)p, (slot0 + i) % b.n_arms, 1u, acc);
            frames_out[i] = f;
        }
    } else {
        // warp-uniform trip count (blockDim is a multiple of 32), so the warp
        // can merge the pins of lanes fetching the same page
        const uint32_t lane = threadIdx.x & 31u;
        for (uint64_t base = tid - lane; base < n; base += nthr) {
            const uint64_t i = base + lane;
            const int32_t p = i < n ? pages[i] : -1;
            const bool valid = p >= 0 && (uint32_t)p < b.n_logical;
            const uint32_t key = valid ? (uint32_t)p : 0x80000000u + lane;   // invalid lanes never merge
            const uint32_t peers = __match_any_sync(0xffffffffu, key);
            const uint32_t leader = (uint32_t)__ffs((int)peers) - 1u;
            int32_t hit = -1, f0 = kLoading;
            if (valid && lane == leader) {
                f0 = __ldcg(b.page_table + p);
                if (f0 >= 0 && pin_if_owner(b, f0, (uint32_t)p, (uint32_t)__popc(peers))) {
                    b.ref[f0] = 1;
                    hit = f0;
                }
            }
            hit = __shfl_sync(0xffffffffu, hit, (int)leader);
            int32_t f = -1;
            bool loader = false;
            if constexpr (!DIST) {
                // single hand: the leaders of pages that are not resident become
                // their loaders and sweep together; the other lanes fetch as below
                // (their pages are resident, or being loaded, by then)
                if (hit < 0 && valid && lane == leader)
                    loader = f0 == -1 && atomicCAS(b.page_table + p, -1, kLoading) == -1;
                const uint32_t lm = __ballot_sync(0xffffffffu, loader);
                if (lm) {
                    uint32_t old_page = kEmptyPage;
                    const int32_t h = sweep_warp(b, lm, (uint32_t)p, &old_page);
                    finish_loads_warp(b, loader, (uint32_t)p, h, old_page, acc);
                    if (loader) f = h;
                }
            }
            if (hit >= 0) {
                f = hit;
                ++acc.hits;
            } else if (valid && !loader) {
                f = fetch<DIST>(b, (uint32_t)p, (slot0 + (uint32_t)i) % b.n_arms, kHandBatch, acc);
            }
            if (i < n) frames_out[i] = f;
        }
    }
    block_add_counters<7>({ok, bad, acc.hits, acc.misses, acc.evictions, acc.failures, acc.timeouts},
                          {&b.stats->unpins, &b.stats->bad_unpins, &b.stats->hits, &b.stats->misses,
                           &b.stats->evictions, &b.stats->failures, &b.stats->timeouts});
}

__global__ void k_bm_init(BmView b) {
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t nthr = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t p = tid; p < b.n_logical; p += nthr) b.page_table[p] = -1;
    for (uint64_t f = tid; f < b.n_frames; f += nthr) {
        b.frame_state[f] = (unsigned long long)kEmptyPage << 32;
        b.ref[f] = 0;
    }
    for (uint64_t a = tid; a < b.n_arms; a += nthr)
        b.arms[a] = (uint32_t)(((unsigned long long)a * b.n_frames) / b.n_arms);
    if (tid == 0) *b.single_hand = 0ull;
}

// Consistency check: page_table and frame_state are inverse maps; pins sum.
struct BmCheck {
    unsigned long long resident, mapped_frames, mismatches, loading, pins;
};

__global__ void k_bm_check(BmView b, BmCheck* out) {
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t nthr = (uint64_t)gridDim.x * blockDim.x;
    unsigned long long res = 0, mapped = 0, mism = 0, loading = 0, pins = 0;
    for (uint64_t p = tid; p < b.n_logical; p += nthr) {
        int32_t f = b.page_table[p];
        if (f == kLoading) { ++loading; continue; }
        if (f < 0) continue;
        ++res;
        if ((uint32_t)f >= b.n_frames || (uint32_t)(b.frame_state[f] >> 32) != p) ++mism;
    }
    for (uint64_t f = tid; f < b.n_frames; f += nthr) {
        unsigned long long s = b.frame_state[f];
        uint32_t pg = (uint32_t)(s >> 32);
        pins += (uint32_t)s;
        if (pg == kEmptyPage) continue;
        ++mapped;
        if (pg >= b.n_logical || b.page_table[pg] != (int32_t)f) ++mism;
    }
    if (res) atomicAdd(&out->resident, res);
    if (mapped) atomicAdd(&out->mapped_frames, mapped);
    if (mism) atomicAdd(&out->mismatches, mism);
    if (loading) atomicAdd(&out->loading, loading);
    if (pins) atomicAdd(&out->pins, pins);
}

__global__ void k_bm_gather(BmView b, const int32_t* ids, uint32_t n, uint32_t words_per_frame, int32_t* out) {
    const unsigned long long total = (unsigned long long)n * words_per_frame;
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        uint32_t r = (uint32_t)(i / words_per_frame), k = (uint32_t)(i % words_per_frame);
        int32_t f = ids[r];
        out[i] = (f >= 0 && (uint32_t)f < b.n_frames)
                     ? reinterpret_cast<const int32_t*>(b.frames + (size_t)(uint32_t)f * b.frame_size)[k]
                     : 0;
    }
}

}  // namespace
}  // namespace pbm

using namespace pbm;

struct pbm_bufmgr {
    BmView v;
    BmCheck* d_check;
    size_t frames_bytes;
};

extern "C" {

int pbm_bufmgr_create(const pbm_bufmgr_config* cfg, const void* d_backing, pbm_bufmgr** out) {
    if (!cfg || !out || cfg->n_logical == 0 || cfg->n_logical > 0x7fffffffull || cfg->n_frames == 0 ||
        cfg->n_frames >= 0x7fffffffu || (cfg->frame_size % 16u) != 0 || cfg->policy < 0 || cfg->policy > 1)
        return PBM_ERR_INVALID;
    *out = nullptr;
    pbm_bufmgr* m = new (std::nothrow) pbm_bufmgr();
    if (!m) return PBM_ERR_NOMEM;
    std::memset((void*)m, 0, sizeof(*m));
    BmView& b = m->v;
    b.n_logical = (uint32_t)cfg->n_logical;
    b.n_frames = cfg->n_frames;
    b.frame_size = cfg->frame_size;
    b.max_sweep = cfg->max_sweep ? cfg->max_sweep : 2u * cfg->n_frames + 64u;
    b.n_arms = cfg->n_arms ? cfg->n_arms : 1u;
    b.dist = cfg->policy;
    b.backing = (const char*)d_backing;
    bool ok = cudaMalloc(&b.page_table, sizeof(int32_t) * b.n_logical) == cudaSuccess &&
              cudaMalloc(&b.frame_state, sizeof(unsigned long long) * b.n_frames) == cudaSuccess &&
              cudaMalloc(&b.ref, b.n_frames) == cudaSuccess &&
              cudaMalloc(&b.single_hand, sizeof(unsigned long long)) == cudaSuccess &&
              cudaMalloc(&b.arms, sizeof(uint32_t) * b.n_arms) == cudaSuccess &&
              cudaMalloc(&b.stats, sizeof(BmStats)) == cudaSuccess &&
              cudaMalloc(&m->d_check, sizeof(BmCheck)) == cudaSuccess;
    if (ok && cfg->frame_size) {
        m->frames_bytes = (size_t)b.n_frames * cfg->frame_size;
        ok = cudaMalloc(&b.frames, m->frames_bytes) == cudaSuccess;
    }
    if (!ok) {
        cudaGetLastError();
        pbm_bufmgr_destroy(m);
        return PBM_ERR_NOMEM;
    }
    int rc = pbm_bufmgr_reset(m, nullptr);
    if (rc == PBM_OK && cudaDeviceSynchronize() != cudaSuccess) rc = PBM_ERR_CUDA;
    if (rc) { pbm_bufmgr_destroy(m); return rc; }
    *out = m;
    return PBM_OK;
}

int pbm_bufmgr_destroy(pbm_bufmgr* m) {
    if (!m) return PBM_ERR_INVALID;
    cudaDeviceSynchronize();
    cudaFree(m->v.page_table);
    cudaFree(m->v.frame_state);
    cudaFree(m->v.ref);
    cudaFree(m->v.single_hand);
    cudaFree(m->v.arms);
    cudaFree(m->v.stats);
    cudaFree(m->v.frames);
    cudaFree(m->d_check);
    delete m;
    return PBM_OK;
}

int pbm_bufmgr_reset(pbm_bufmgr* m, void* stream) {
    if (!m) return PBM_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    k_bm_init<<<sm_count() * 4, 256, 0, s>>>(m->v);
    PBM_LAUNCH_CHECK();
    PBM_CUDA_TRY(cudaMemsetAsync(m->v.stats, 0, sizeof(BmStats), s));
    return PBM_OK;
}

int pbm_bufmgr_round(pbm_bufmgr* m, const int32_t* d_frames_of, const int32_t* d_release_idx,
                     uint32_t n_release, const int32_t* d_pages, uint32_t n, uint32_t slot0,
                     int32_t* d_frames_out, int serial, void* stream) {
    if (!m || (n_release && (!d_frames_of || !d_release_idx)) || (n && (!d_pages || !d_frames_out)))
        return PBM_ERR_INVALID;
    if (n == 0 && n_release == 0) return PBM_OK;
    const uint32_t work = n > n_release ? n : n_release;
    int block = serial ? 1 : 256;
    int grid = serial ? 1 : (int)((work + 255u) / 256u);
    if (m->v.dist)
        k_round<true><<<grid, block, 0, (cudaStream_t)stream>>>(m->v, d_frames_of, d_release_idx, n_release,
                                                                d_pages, n, slot0, d_frames_out);
    else
        k_round<false><<<grid, block, 0, (cudaStream_t)stream>>>(m->v, d_frames_of, d_release_idx, n_release,
                                                                 d_pages, n, slot0, d_frames_out);
    PBM_LAUNCH_CHECK();
    return PBM_OK;
}

int pbm_bufmgr_stats(pbm_bufmgr* m, pbm_bufmgr_counters* h_out, void* stream) {
    if (!m || !h_out) return PBM_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    BmStats d;
    PBM_CUDA_TRY(cudaMemcpyAsync(&d, m->v.stats, sizeof(d), cudaMemcpyDeviceToHost, s));
    PBM_CUDA_TRY(cudaStreamSynchronize(s));
    h_out->hits = d.hits;
    h_out->misses = d.misses;
    h_out->evictions = d.evictions;
    h_out->failures = d.failures;
    h_out->unpins = d.unpins;
    h_out->bad_unpins = d.bad_unpins;
    h_out->timeouts = d.timeouts;
    return (d.timeouts || d.bad_unpins) ? PBM_ERR_CORRUPT : PBM_OK;
}

int pbm_bufmgr_check(pbm_bufmgr* m, pbm_bufmgr_check_result* h_out, void* stream) {
    if (!m || !h_out) return PBM_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    PBM_CUDA_TRY(cudaMemsetAsync(m->d_check, 0, sizeof(BmCheck), s));
    k_bm_check<<<sm_count() * 4, 256, 0, s>>>(m->v, m->d_check);
    PBM_LAUNCH_CHECK();
    BmCheck c;
    PBM_CUDA_TRY(cudaMemcpyAsync(&c, m->d_check, sizeof(c), cudaMemcpyDeviceToHost, s));
    PBM_CUDA_TRY(cudaStreamSynchronize(s));
    h_out->resident = c.resident;
    h_out->mapped_frames = c.mapped_frames;
    h_out->mismatches = c.mismatches;
    h_out->loading = c.loading;
    h_out->pins = c.pins;
    return (c.mismatches || c.loading || c.resident != c.mapped_frames) ? PBM_ERR_CORRUPT : PBM_OK;
}

int pbm_bufmgr_gather(pbm_bufmgr* m, const int32_t* d_frame_ids, uint32_t n, uint32_t bytes_per_frame,
                      int32_t* d_out, void* stream) {
    if (!m || !m->v.frames || (n && (!d_frame_ids || !d_out)) || bytes_per_frame == 0 ||
        bytes_per_frame > m->v.frame_size || (bytes_per_frame & 3u))
        return PBM_ERR_INVALID;
    if (n == 0) return PBM_OK;
    k_bm_gather<<<sm_count() * 4, 256, 0, (cudaStream_t)stream>>>(m->v, d_frame_ids, n, bytes_per_frame / 4u,
                                                                  d_out);
    PBM_LAUNCH_CHECK();
    return PBM_OK;
}

int pbm_bufmgr_frames(pbm_bufmgr* m, void** d_frames, size_t* bytes) {
    if (!m) return PBM_ERR_INVALID;
    if (d_frames) *d_frames = m->v.frames;
    if (bytes) *bytes = m->frames_bytes;
    return PBM_OK;
}

}  // extern "C"
