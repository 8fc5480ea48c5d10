// pbm_device.cuh -- device-side core of the GB300 page manager.
//
// Everything a kernel needs to allocate and free pages of a pool from any
// thread: the pool descriptor, the reference's LCG, the index mapping, and
// the walks (per-thread page probe, per-thread word probe, warp-collaborative
// walk, clustered walk, clock sweeps, contiguous runs) plus frees.
//
// The same inline routines run inside this library's batch kernels and in a
// caller's own kernels through the drop-in headers (RandomWalkBasic.cuh,
// RandomWalkBasic_BM.cuh, CollabRW_BM.cuh, CRW_BM.cuh, RWMalloc.cuh,
// parallelPage.cuh).
//
// Bitmap layout: bit b of 32-bit word w <-> page 32*w + b; bit set = held.
// The 64-bit view reads the same bytes (page 64*w + b), so the storage is
// padded to an even number of 32-bit words and every bit past the last page
// is kept set.  All walks are bounded: after max_steps random jumps a
// request returns -1 instead of trapping or spinning.
#pragma once
#include <cstdint>

namespace pbm {

// Pool descriptor, passed by value (or read from a __device__ global by the
// drop-in API).  32 bytes.
struct PoolView {
    uint32_t* words;      // bitmap, n_words32 (even) 32-bit words
    char*     base;       // page memory (pageAddress), may be null
    uint32_t  n_pages;    // T
    uint32_t  n_words32;  // ceil(T/32)
    uint32_t  n_words64;  // ceil(T/64)
    uint32_t  page_size;  // bytes
};

// Device statistics block (one per pool), updated with block-aggregated atomics.
struct DevStats {
    unsigned long long successes;
    unsigned long long failures;
    unsigned long long steps;
    unsigned long long frees;
    unsigned long long timeouts;   // bounded waits that gave up
    unsigned long long bad_frees;  // malloc frees rejected (outside the pool / double free)
    unsigned long long pad[2];
};

// FIFO free list of the linked-list strategy: a ring of page ids with
// ticket counters.  `avail` is a signed count stored in two's complement.
// Every get and put of every thread hits these counters, so each has a
// 128-byte line (an L2 slice's atomic unit) of its own.
struct FifoState {
    alignas(128) unsigned long long head;    // next get ticket
    alignas(128) unsigned long long tail;    // next put ticket
    alignas(128) unsigned long long avail;   // free pages in the ring
};

constexpr uint32_t kFifoSpinLimit = 1u << 20;   // bounded waits in the free list
constexpr uint32_t kFull32 = 0xffffffffu;
constexpr uint64_t kFull64 = 0xffffffffffffffffull;

// ---------------------------------------------------------------------------
// RNG
// ---------------------------------------------------------------------------

// source/RNG_LCG.cuh:9-12: (1103515245*x + 12345) % (1<<31) in signed 64-bit
// with C truncation, cast to int.  The remainder by 2^31 is a mask of the
// magnitude, so no 64-bit division is issued.
__host__ __device__ __forceinline__ int32_t lcg(int32_t x) {
    long long v = 1103515245LL * (long long)x + 12345LL;
    long long r = v >= 0 ? (v & 0x7fffffffLL) : -((-v) & 0x7fffffffLL);
    return (int32_t)r;
}

// The same step for a state in [0, 2^31), which is every state the walks
// see (request seeds are 31-bit and the LCG keeps non-negative states
// non-negative): (A*x + C) mod 2^31 is then the low 31 bits of the 32-bit
// product, so one multiply-add and a mask replace the 64-bit arithmetic.
__host__ __device__ __forceinline__ int32_t lcg31(int32_t x) {
    return (int32_t)((1103515245u * (uint32_t)x + 12345u) & 0x7fffffffu);
}

// Index in [0, n) from the LCG state's 31 bits by multiply-high.  The
// reference reduces with `(unsigned)x % n`; for power-of-two n that keeps
// only the LCG's low bits, whose short periods make threads with equal low
// seed bits walk identical sequences.  The high bits do not have that flaw.
__host__ __device__ __forceinline__ uint32_t idx_hi(int32_t x, uint32_t n) {
    return (uint32_t)((((unsigned long long)((uint32_t)x & 0x7fffffffu)) * n) >> 31);
}

// Per-request seed: murmur3 fmix32 of (stream seed, request index), 31 bits.
__host__ __device__ __forceinline__ int32_t request_seed(uint32_t S, uint32_t r) {
    uint32_t h = r * 0x9E3779B1u + S * 0x85EBCA77u + 0x165667B1u;
    h ^= h >> 16; h *= 0x85EBCA6Bu;
    h ^= h >> 13; h *= 0xC2B2AE35u;
    h ^= h >> 16;
    return (int32_t)(h & 0x7fffffffu);
}

// splitmix64 output function on a Weyl counter (Bernoulli prefill).
__host__ __device__ __forceinline__ uint64_t hash64(uint64_t seed, uint64_t ctr) {
    uint64_t z = seed * 0xD1B54A32D192ED03ull + (ctr + 1ull) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

#ifdef __CUDACC__

// ---------------------------------------------------------------------------
// Word access
// ---------------------------------------------------------------------------

// Bitmap loads bypass L1 (it is not coherent with the L2 atomics); a stale
// value would only waste a probe, the atomic stays authoritative.
__device__ __forceinline__ uint32_t load_word(const uint32_t* p) { return __ldcg(p); }
__device__ __forceinline__ uint64_t load_word(const uint64_t* p) {
    return (uint64_t)__ldcg(reinterpret_cast<const unsigned long long*>(p));
}
__device__ __forceinline__ uint32_t atomic_or(uint32_t* p, uint32_t m) { return atomicOr(p, m); }
__device__ __forceinline__ uint64_t atomic_or(uint64_t* p, uint64_t m) {
    return (uint64_t)atomicOr(reinterpret_cast<unsigned long long*>(p), (unsigned long long)m);
}
__device__ __forceinline__ void atomic_and_noret(uint32_t* p, uint32_t m) { atomicAnd(p, m); }
__device__ __forceinline__ void atomic_and_noret(uint64_t* p, uint64_t m) {
    atomicAnd(reinterpret_cast<unsigned long long*>(p), (unsigned long long)m);
}
__device__ __forceinline__ int popc_w(uint32_t x) { return __popc(x); }
__device__ __forceinline__ int popc_w(uint64_t x) { return __popcll(x); }
__device__ __forceinline__ int ctz_w(uint32_t x) { return __ffs((int)x) - 1; }
__device__ __forceinline__ int ctz_w(uint64_t x) { return __ffsll((long long)x) - 1; }

// Position of the (k+1)-th set bit of m (0 <= k < popc(m)): five halving
// steps, each counting the set bits of the lower half and moving into the
// upper half when k lies beyond them (branch-free, no loop; measured faster
// than __fns in the walks).
__device__ __forceinline__ uint32_t nth_set_bit(uint32_t m, int k) {
    uint32_t pos = 0;
    int c = __popc(m & 0xffffu);
    if (k >= c) { k -= c; pos += 16u; m >>= 16; }
    c = __popc(m & 0xffu);
    if (k >= c) { k -= c; pos += 8u; m >>= 8; }
    c = __popc(m & 0xfu);
    if (k >= c) { k -= c; pos += 4u; m >>= 4; }
    c = __popc(m & 0x3u);
    if (k >= c) { k -= c; pos += 2u; m >>= 2; }
    if (k >= (int)(m & 1u)) pos += 1u;
    return pos;
}

// Lowest k set bits of m (0 <= k <= popc(m)).
__device__ __forceinline__ uint32_t low_bits(uint32_t m, int k) {
    if (k <= 0) return 0u;
    if (k >= __popc(m)) return m;
    return m & ((1u << nth_set_bit(m, k)) - 1u);   // below the (k+1)-th set bit
}
__device__ __forceinline__ uint64_t low_bits(uint64_t m, int k) {
    if (k <= 0) return 0ull;
    uint32_t lo = (uint32_t)m, hi = (uint32_t)(m >> 32);
    int clo = __popc(lo);
    if (k <= clo) return (uint64_t)low_bits(lo, k);
    return (uint64_t)lo | ((uint64_t)low_bits(hi, k - clo) << 32);
}

template <typename Word> struct WordTraits;
template <> struct WordTraits<uint32_t> {
    static constexpr int kBits = 32;
    static constexpr int kShift = 5;
    __device__ static uint32_t full() { return kFull32; }
    __device__ static uint32_t count(const PoolView& v) { return v.n_words32; }
};
template <> struct WordTraits<uint64_t> {
    static constexpr int kBits = 64;
    static constexpr int kShift = 6;
    __device__ static uint64_t full() { return kFull64; }
    __device__ static uint32_t count(const PoolView& v) { return v.n_words64; }
};

// ---------------------------------------------------------------------------
// Per-thread page-probe walk (RandomWalkBasic semantics, on the bitmap):
// probe a random page with one atomicOr of its bit, which takes the page
// when the bit was clear and changes nothing when it was set (the reference
// exchanges each probed map entry, source/RandomWalkBasic.cuh:54-74); steps =
// probes.  One round trip per probe.  Measured on GB300 (churn at 50 / 75 /
// 90 / 95% occupancy): 54 / 30 / 13 / 6.9 G ops/s against 37 / 21 / 11 / 6.7
// reading the word first; only walks that run to their bound in an exhausted
// pool pay for it, with an atomic instead of a load per missed probe.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int32_t walk_page(const PoolView& v, int32_t seed0,
                                             uint32_t max_steps, int32_t* steps_out) {
    int32_t x = seed0 & 0x7fffffff;   // walks run on 31-bit states
    uint32_t s = 0;
    while (s < max_steps) {
        ++s;
        x = lcg31(x);
        uint32_t p = idx_hi(x, v.n_pages);
        uint32_t* wp = v.words + (p >> 5);
        uint32_t bit = 1u << (p & 31u);
        const uint32_t old = atomicOr(wp, bit);
        if (!(old & bit)) {
            if (steps_out) *steps_out = (int32_t)s;
            return (int32_t)p;
        }
    }
    if (steps_out) *steps_out = (int32_t)s;
    return -1;
}

// ---------------------------------------------------------------------------
// Per-thread word-probe walk (RandomWalkBasic_BM semantics): jump to a random
// word, claim its lowest clear bit; on a lost race retry in the same word;
// steps = jumps.  source/RandomWalkBasic_BM.cuh:60-89.  (Taking every clear
// bit with one atomicOr of all ones and handing the rest back is one round
// trip instead of two, but a racer that jumps to a word while its bits are
// held sees it full and jumps again: measured on GB300, 7% more jumps with
// 4,096 walkers on 32,768 words, outside the word-probe model's 3-SE band;
// the collaborative walks use it, where the gain is measured and the model
// still holds.)
// ---------------------------------------------------------------------------
template <typename Word>
__device__ __forceinline__ int32_t walk_word(const PoolView& v, int32_t seed0,
                                             uint32_t max_steps, int32_t* steps_out) {
    using T = WordTraits<Word>;
    Word* words = reinterpret_cast<Word*>(v.words);
    const uint32_t L = T::count(v);
    int32_t x = seed0 & 0x7fffffff;   // walks run on 31-bit states
    uint32_t s = 0;
    while (s < max_steps) {
        ++s;
        x = lcg31(x);
        uint32_t w = idx_hi(x, L);
        Word val = load_word(words + w);
        while (val != T::full()) {
            int b = ctz_w((Word)~val);
            Word bit = (Word)1 << b;
            Word old = atomic_or(words + w, bit);
            if (!(old & bit)) {
                if (steps_out) *steps_out = (int32_t)s;
                return (int32_t)(((uint32_t)w << T::kShift) + (uint32_t)b);
            }
            val = old | bit;
        }
    }
    if (steps_out) *steps_out = (int32_t)s;
    return -1;
}

// ---------------------------------------------------------------------------
// Warp-collaborative walk (CollabRW_BM, source/CollabRW_BM.cuh:114-160,
// restated lock-free).  A group of W lanes (W = 8, 16 or 32, aligned within
// the warp) shares one LCG stream.  Per jump lane i takes word
// (base + i*stride) mod L -- one cache line for the group when stride == 1 --
// with one atomicOr of all ones: the read and the claim of every clear bit
// of the word in a single round trip, as the reference grabs whole words.
// The group keeps as many of those bits as it still needs -- lowest lanes
// and lowest bits first -- and hands the rest straight back with one
// atomicAnd per word (the reference writes whole words back with atomicExch,
// which drops pages freed meanwhile; an AND of exactly the surplus cannot).
// The kept bits go to the needing lanes in lane order (needing lane of rank
// r takes the r-th kept bit).  Needs left unmet go to the next jump.  Every
// bit a lane takes is its own, so no claim is ever lost to a concurrent one;
// surplus bits are held only between the two atomics, and a walker that
// reads them in that window skips them.  (Reading the words first and then
// claiming only the planned bits costs a second dependent round trip per
// jump; on GB300 the single grab is 5-7% faster at 90% occupancy.)
// Lanes whose words coincide (only possible when W*stride > L): only the
// lowest of them grabs (__match_any_sync), so every word is taken once and
// the result is that of lane order.
//
// Every lane of the group must call this converged; `need` says whether the
// lane requests a page.  All lanes of the group report the same step count
// (jumps of the group), as in the reference.  `slots` is unused (kept for
// the callers' shared scratch layout).
// ---------------------------------------------------------------------------
template <int W>
__device__ __forceinline__ int group_incl_scan(int v, uint32_t gl, uint32_t gmask) {
#pragma unroll
    for (int d = 1; d < W; d <<= 1) {
        int y = __shfl_up_sync(gmask, v, d, W);
        if ((int)gl >= d) v += y;
    }
    return v;
}

// Position of the (k+1)-th set bit of m (k < popc(m)).
__device__ __forceinline__ uint32_t nth_bit(uint32_t m, int k) { return nth_set_bit(m, k); }
__device__ __forceinline__ uint32_t nth_bit(uint64_t m, int k) {
    const uint32_t lo = (uint32_t)m;
    const int c = __popc(lo);
    return k < c ? nth_set_bit(lo, k) : 32u + nth_set_bit((uint32_t)(m >> 32), k - c);
}

template <int W, typename Word>
__device__ __forceinline__ int32_t walk_collab(const PoolView& v, bool need, int32_t group_seed,
                                               uint32_t lane_off /* (lane_in_group*stride) % L */,
                                               bool dedupe, uint32_t max_steps,
                                               volatile int32_t* slots, int32_t* steps_out) {
    (void)slots;
    using T = WordTraits<Word>;
    Word* words = reinterpret_cast<Word*>(v.words);
    const uint32_t L = T::count(v);
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t gl = lane & (uint32_t)(W - 1);                    // lane in group
    const uint32_t gmask = (W == 32) ? kFull32 : (((1u << W) - 1u) << (lane & ~(uint32_t)(W - 1)));
    const uint32_t lt = (1u << lane) - 1u;                           // lanes below me
    int32_t id = -1;
    int32_t x = group_seed & 0x7fffffff;
    uint32_t needm = __ballot_sync(gmask, need);
    uint32_t s = 0;
    while (needm && s < max_steps) {
        ++s;
        x = lcg31(x);
        uint32_t w = idx_hi(x, L) + lane_off;
        if (w >= L) w -= L;
        bool grab = true;
        if (dedupe) grab = (__match_any_sync(gmask, w) & lt) == 0u;   // a lower lane takes this word
        const Word fr = grab ? (Word)~atomic_or(words + w, T::full()) : (Word)0;
        {
            const int cnt = popc_w(fr);
            const int incl = group_incl_scan<W>(cnt, gl, gmask);
            const int n = __popc(needm);
            const Word got = low_bits(fr, n - (incl - cnt));        // kept: the first n in lane order
            const Word extra = fr & (Word)~got;
            if (extra) atomic_and_noret(words + w, (Word)~extra);   // surplus handed back
            const int g = popc_w(got);
            // inclusive prefix of the kept bits, and their total
            const int gincl = min(incl, n);
            const int G = min(__shfl_sync(gmask, incl, W - 1, W), n);
            if (G > 0) {
                // needing lane of rank r takes gained bit r: its source is the
                // first group lane whose inclusive gain exceeds r
                const int r = need && id < 0 ? __popc(needm & lt) : 0;
                int src = 0;
#pragma unroll
                for (int step = W / 2; step >= 1; step >>= 1) {
                    const int gv = __shfl_sync(gmask, gincl, src + step - 1, W);
                    if (gv <= r) src += step;
                }
                const int src_excl = __shfl_sync(gmask, gincl - g, src, W);
                const uint32_t src_w = __shfl_sync(gmask, w, src, W);
                Word src_got;
                if constexpr (sizeof(Word) == 8) {
                    const uint32_t lo = __shfl_sync(gmask, (uint32_t)got, src, W);
                    const uint32_t hi = __shfl_sync(gmask, (uint32_t)(got >> 32), src, W);
                    src_got = ((Word)hi << 32) | (Word)lo;
                } else {
                    src_got = __shfl_sync(gmask, got, src, W);
                }
                if (need && id < 0 && r < G)
                    id = (int32_t)((src_w << T::kShift) + nth_bit(src_got, r - src_excl));
            }
            needm = __ballot_sync(gmask, need && id < 0);
        }
    }
    if (steps_out) *steps_out = (int32_t)s;
    return id;
}

// ---------------------------------------------------------------------------
// The collaborative walk for two requests per lane (a warp serving 64
// requests at a time): the same jump, window, plan and atomics as
// walk_collab<32, Word>, with the needing requests ranked a-requests first
// (lane order), then b-requests; request of rank r takes gained bit r.  The
// jump's fixed costs (window load, scan, claims) are shared by up to 64
// requests.  The whole warp calls converged.
// ---------------------------------------------------------------------------
template <typename Word>
__device__ __forceinline__ void collab_take(int r, int gincl, int g, uint32_t w, Word got, int32_t& id) {
    using T = WordTraits<Word>;
    int src = 0;
#pragma unroll
    for (int step = 16; step >= 1; step >>= 1) {
        const int gv = __shfl_sync(kFull32, gincl, src + step - 1);
        if (gv <= r) src += step;
    }
    const int src_excl = __shfl_sync(kFull32, gincl - g, src);
    const uint32_t src_w = __shfl_sync(kFull32, w, src);
    Word src_got;
    if constexpr (sizeof(Word) == 8) {
        const uint32_t lo = __shfl_sync(kFull32, (uint32_t)got, src);
        const uint32_t hi = __shfl_sync(kFull32, (uint32_t)(got >> 32), src);
        src_got = ((Word)hi << 32) | (Word)lo;
    } else {
        src_got = __shfl_sync(kFull32, got, src);
    }
    id = (int32_t)((src_w << T::kShift) + nth_bit(src_got, r - src_excl));
}

template <typename Word>
__device__ __forceinline__ void walk_collab2(const PoolView& v, bool need_a, bool need_b, int32_t group_seed,
                                             uint32_t lane_off, bool dedupe, uint32_t max_steps, int32_t& id_a,
                                             int32_t& id_b, int32_t* steps_out) {
    using T = WordTraits<Word>;
    Word* words = reinterpret_cast<Word*>(v.words);
    const uint32_t L = T::count(v);
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t lt = (1u << lane) - 1u;
    id_a = -1;
    id_b = -1;
    int32_t x = group_seed & 0x7fffffff;
    uint32_t ma = __ballot_sync(kFull32, need_a), mb = __ballot_sync(kFull32, need_b);
    uint32_t s = 0;
    while ((ma | mb) && s < max_steps) {
        ++s;
        x = lcg31(x);
        uint32_t w = idx_hi(x, L) + lane_off;
        if (w >= L) w -= L;
        bool grab = true;
        if (dedupe) grab = (__match_any_sync(kFull32, w) & lt) == 0u;   // a lower lane takes this word
        const Word fr = grab ? (Word)~atomic_or(words + w, T::full()) : (Word)0;
        const int cnt = popc_w(fr);
        const int incl = group_incl_scan<32>(cnt, lane, kFull32);
        const int na = __popc(ma);
        const int n = na + __popc(mb);
        const Word got = low_bits(fr, n - (incl - cnt));
        const Word extra = fr & (Word)~got;
        if (extra) atomic_and_noret(words + w, (Word)~extra);
        const int g = popc_w(got);
        const int gincl = min(incl, n);
        const int G = min(__shfl_sync(kFull32, incl, 31), n);
        if (G > 0) {
            const bool wa = need_a && id_a < 0, wb = need_b && id_b < 0;
            const int ra = wa ? __popc(ma & lt) : 0;
            const int rb = wb ? na + __popc(mb & lt) : 0;
            int32_t ta = -1, tb = -1;
            collab_take<Word>(ra, gincl, g, w, got, ta);
            if (__any_sync(kFull32, wb && rb < G)) collab_take<Word>(rb, gincl, g, w, got, tb);
            if (wa && ra < G) id_a = ta;
            if (wb && rb < G) id_b = tb;
        }
        ma = __ballot_sync(kFull32, need_a && id_a < 0);
        mb = __ballot_sync(kFull32, need_b && id_b < 0);
    }
    if (steps_out) *steps_out = (int32_t)s;
}

// ---------------------------------------------------------------------------
// The collaborative walk over an arbitrary set of converged lanes `active`
// (the drop-in form: the reference's getPage runs on __activemask(),
// CollabRW_BM.cuh:119).  Active lane k (k-th set bit of `active`) takes word
// (base + k) mod L with the same grab and hand-back as walk_collab; prefix
// sums use bit-sliced ballots, so inactive lanes never participate.  `slots`
// = 32 ints of shared memory for this warp.
// ---------------------------------------------------------------------------
template <typename Word>
__device__ __forceinline__ int32_t walk_collab_masked(const PoolView& v, uint32_t active, bool need,
                                                      int32_t seed, uint32_t max_steps,
                                                      volatile int32_t* slots, int32_t* steps_out) {
    using T = WordTraits<Word>;
    Word* words = reinterpret_cast<Word*>(v.words);
    const uint32_t L = T::count(v);
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t lt = (1u << lane) - 1u;
    const uint32_t k = (uint32_t)__popc(active & lt);
    const uint32_t off = k % L;
    const bool dedupe = __popc(active) > (int)L;
    int32_t id = -1;
    int32_t x = seed & 0x7fffffff;
    uint32_t needm = __ballot_sync(active, need);
    uint32_t s = 0;
    while (needm && s < max_steps) {
        ++s;
        x = lcg31(x);
        uint32_t w = idx_hi(x, L) + off;
        if (w >= L) w -= L;
        bool grab = true;
        if (dedupe) grab = (__match_any_sync(active, w) & lt) == 0u;   // a lower lane takes this word
        const Word fr = grab ? (Word)~atomic_or(words + w, T::full()) : (Word)0;
        int cnt = popc_w(fr);
        int pre = 0;
#pragma unroll
        for (int b = 0; b < 7; ++b) pre += __popc(__ballot_sync(active, (cnt >> b) & 1) & lt) << b;
        int n = __popc(needm);
        Word got = low_bits(fr, n - pre);                            // kept; the surplus goes back
        const Word extra = fr & (Word)~got;
        if (extra) atomic_and_noret(words + w, (Word)~extra);
        int g = popc_w(got);
        int gpre = 0, G = 0;
#pragma unroll
        for (int b = 0; b < 7; ++b) {
            uint32_t bm = __ballot_sync(active, (g >> b) & 1);
            gpre += __popc(bm & lt) << b;
            G += __popc(bm) << b;
        }
        int pos = gpre;
        while (got) {
            int b = ctz_w(got);
            got &= got - (Word)1;
            slots[pos++] = (int32_t)(((uint32_t)w << T::kShift) + (uint32_t)b);
        }
        __syncwarp(active);
        if (id < 0 && need) {
            int rank = __popc(needm & lt);
            if (rank < G) id = slots[rank];
        }
        __syncwarp(active);
        needm = __ballot_sync(active, need && id < 0);
    }
    if (steps_out) *steps_out = (int32_t)s;
    return id;
}

// ---------------------------------------------------------------------------
// Clustered walk (CRW_BM, source/CRW_BM.cuh:75-142): resume at the word of
// this slot's last page (the next word once the last page was the word's
// top bit) and claim its lowest clear bit; otherwise random word-probe
// jumps.  steps = claim attempts (the reference does not count jumps).
// `cursor` = last page of the slot or -1; updated on success.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int32_t walk_crw(const PoolView& v, int32_t* cursor, int32_t seed0,
                                            uint32_t max_steps, int32_t* steps_out) {
    const uint32_t L = v.n_words32;
    int32_t s = 0;
    int32_t last = *cursor;
    if (last >= 0) {
        uint32_t w = (uint32_t)last >> 5;
        if (((uint32_t)last & 31u) == 31u) { w += 1u; if (w == L) w = 0; }
        uint32_t val = load_word(v.words + w);
        while (val != kFull32) {
            ++s;
            int b = __ffs((int)~val) - 1;
            uint32_t bit = 1u << b;
            uint32_t old = atomicOr(v.words + w, bit);
            if (!(old & bit)) {
                *cursor = (int32_t)(w * 32u + (uint32_t)b);
                if (steps_out) *steps_out = s;
                return *cursor;
            }
            val = old | bit;
        }
    }
    int32_t x = seed0 & 0x7fffffff;   // walks run on 31-bit states
    for (uint32_t j = 0; j < max_steps; ++j) {
        x = lcg31(x);
        uint32_t w = idx_hi(x, L);
        uint32_t val = load_word(v.words + w);
        while (val != kFull32) {
            ++s;
            int b = __ffs((int)~val) - 1;
            uint32_t bit = 1u << b;
            uint32_t old = atomicOr(v.words + w, bit);
            if (!(old & bit)) {
                *cursor = (int32_t)(w * 32u + (uint32_t)b);
                if (steps_out) *steps_out = s;
                return *cursor;
            }
            val = old | bit;
        }
    }
    if (steps_out) *steps_out = s;
    return -1;
}

// ---------------------------------------------------------------------------
// Clock sweeps.  Single clock: one shared arm, atomicAdd then test-and-set
// (parallelPage.cu:491-509 checks and then exchanges without looking at the
// old value; here the claim is the atomicOr's old bit).  Distributed clock:
// a private arm per slot, linear probe (parallelPage.cu:571-592).
// ---------------------------------------------------------------------------
__device__ __forceinline__ int32_t sweep_single(const PoolView& v, unsigned long long* arm,
                                                uint32_t max_steps, int32_t* steps_out) {
    uint32_t s = 0;
    while (s < max_steps) {
        ++s;
        unsigned long long a = atomicAdd(arm, 1ull);
        uint32_t p = (uint32_t)(a % v.n_pages);
        uint32_t* wp = v.words + (p >> 5);
        uint32_t bit = 1u << (p & 31u);
        if (load_word(wp) & bit) continue;
        if (!(atomicOr(wp, bit) & bit)) {
            if (steps_out) *steps_out = (int32_t)s;
            return (int32_t)p;
        }
    }
    if (steps_out) *steps_out = (int32_t)s;
    return -1;
}

__device__ __forceinline__ int32_t sweep_dist(const PoolView& v, uint32_t* arm,
                                              uint32_t max_steps, int32_t* steps_out) {
    uint32_t s = 0, a = *arm;
    int32_t out = -1;
    while (s < max_steps) {
        ++s;
        uint32_t p = a >= v.n_pages ? a - v.n_pages : a;
        a = p + 1u;
        uint32_t* wp = v.words + (p >> 5);
        uint32_t bit = 1u << (p & 31u);
        if (load_word(wp) & bit) continue;
        if (!(atomicOr(wp, bit) & bit)) { out = (int32_t)p; break; }
    }
    *arm = a;
    if (steps_out) *steps_out = (int32_t)s;
    return out;
}

// ---------------------------------------------------------------------------
// Contiguous run of n pages (1..32) inside one 32-bit word, word-probe walk,
// lowest fitting start, claimed with compare-and-swap so a run is either
// taken whole or not at all (parallelPage.cu:1104-1142 sets the bits with
// atomicOr and reverts the wrong ones on a collision; RWMalloc.cuh:203-248).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t run_starts(uint32_t f, uint32_t n) {
    uint32_t r = f, len = 1;
    while (len < n) {
        uint32_t sh = len < n - len ? len : n - len;
        r &= r >> sh;
        len += sh;
    }
    return r;
}

__device__ __forceinline__ int32_t walk_run(const PoolView& v, uint32_t n, int32_t seed0,
                                            uint32_t max_steps, int32_t* steps_out) {
    const uint32_t L = v.n_words32;
    int32_t x = seed0 & 0x7fffffff;   // walks run on 31-bit states
    uint32_t s = 0;
    while (s < max_steps) {
        ++s;
        x = lcg31(x);
        uint32_t w = idx_hi(x, L);
        uint32_t val = load_word(v.words + w);
        for (int tries = 0; tries < 64; ++tries) {
            uint32_t r = run_starts(~val, n);
            if (!r) break;
            uint32_t st = (uint32_t)(__ffs((int)r) - 1);
            uint32_t m = (n >= 32u ? kFull32 : ((1u << n) - 1u)) << st;
            uint32_t old = atomicCAS(v.words + w, val, val | m);
            if (old == val) {
                if (steps_out) *steps_out = (int32_t)s;
                return (int32_t)(w * 32u + st);
            }
            val = old;
        }
    }
    if (steps_out) *steps_out = (int32_t)s;
    return -1;
}

// ---------------------------------------------------------------------------
// Runs that may cross word boundaries (getXPage*_BM / getNPage without the
// one-word limit of parallelPage.cu:1104-1142 and RWMalloc.cuh:203-248).
// Per jump the walk scans words w, w+1, ... (at most ceil(n/32) + 1 of them,
// never past the last word), tracking the free run that reaches the top bit
// of the previous word: a run is found where that run plus the current
// word's free low bits reaches n, or -- for n <= 32 -- inside the current
// word (lowest start).  The run is then claimed word by word with atomicOr;
// if a word had lost some of its bits to another claim, every bit this claim
// set is released again and the walk jumps anew.  steps = jumps.
// ---------------------------------------------------------------------------
constexpr uint32_t kMaxSpanPages = 1u << 16;

// bits lo..hi (inclusive) of a 32-bit word
__host__ __device__ __forceinline__ uint32_t bit_range(uint32_t lo, uint32_t hi) {
    return (hi >= 31u ? kFull32 : ((1u << (hi + 1u)) - 1u)) & ~((1u << lo) - 1u);
}

// mask of the pages of run [p0, p0+n) that lie in word ww
__host__ __device__ __forceinline__ uint32_t span_mask(uint32_t p0, uint32_t n, uint32_t ww) {
    const uint32_t a = p0 >> 5, b = (p0 + n - 1u) >> 5;
    return bit_range(ww == a ? (p0 & 31u) : 0u, ww == b ? ((p0 + n - 1u) & 31u) : 31u);
}

// First run of n <= 32 free pages in words w (value v0) and w+1 (value v1,
// all ones past the last word): inside w, across the boundary, inside w+1.
__device__ __forceinline__ int32_t span_in_pair(uint32_t w, uint32_t v0, uint32_t v1, uint32_t n, uint32_t L) {
    uint32_t r = run_starts(~v0, n);
    if (r) return (int32_t)(w * 32u + (uint32_t)(__ffs((int)r) - 1));
    const uint32_t hi = v0 ? (uint32_t)__clz((int)v0) : 32u;
    if (w + 1u >= L) return -1;
    const uint32_t lo = v1 ? (uint32_t)(__ffs((int)v1) - 1) : 32u;
    if (hi > 0u && hi + lo >= n) return (int32_t)(w * 32u + 32u - hi);
    r = run_starts(~v1, n);
    if (r) return (int32_t)((w + 1u) * 32u + (uint32_t)(__ffs((int)r) - 1));
    return -1;
}

// First run of n free pages seen from word w on (-1 if none in the window).
__device__ __forceinline__ int32_t find_span(const PoolView& v, uint32_t w, uint32_t n) {
    const uint32_t L = v.n_words32;
    if (n <= 32u) {
        // two-word window, both loads in flight together (same result as the loop below)
        const uint32_t v0 = load_word(v.words + w);
        const uint32_t v1 = w + 1u < L ? load_word(v.words + w + 1u) : kFull32;
        return span_in_pair(w, v0, v1, n, L);
    }
    const uint32_t nscan = (n + 31u) / 32u + 1u;
    uint32_t run = 0, start = 0;   // free pages ending at the top of the previous word
    for (uint32_t k = 0; k < nscan && w + k < L; ++k) {
        const uint32_t ww = w + k;
        const uint32_t val = load_word(v.words + ww);
        const uint32_t lo = val ? (uint32_t)(__ffs((int)val) - 1) : 32u;   // free low bits
        if (run > 0u && run + lo >= n) return (int32_t)start;
        if (n <= 32u) {
            const uint32_t r = run_starts(~val, n);
            if (r) return (int32_t)(ww * 32u + (uint32_t)(__ffs((int)r) - 1));
        }
        if (val == 0u) {
            if (run == 0u) start = ww * 32u;
            run += 32u;
        } else {
            const uint32_t hi = (uint32_t)__clz((int)val);            // free top bits
            run = hi;
            start = ww * 32u + 32u - hi;
        }
    }
    return -1;
}

__device__ __forceinline__ void free_span(const PoolView& v, int32_t id, uint32_t n) {
    const uint32_t p0 = (uint32_t)id;
    for (uint32_t ww = p0 >> 5; ww <= (p0 + n - 1u) >> 5; ++ww) atomicAnd(v.words + ww, ~span_mask(p0, n, ww));
}

// Claims the run of n pages at p0 word by word; on a word that lost bits to
// another claim, every bit this claim set is released again.
__device__ __forceinline__ bool claim_span(const PoolView& v, uint32_t p0, uint32_t n) {
    const uint32_t a = p0 >> 5, b = (p0 + n - 1u) >> 5;
    uint32_t ww = a;
    for (; ww <= b; ++ww) {
        const uint32_t m = span_mask(p0, n, ww);
        const uint32_t old = atomicOr(v.words + ww, m);
        if (old & m) {                                   // lost part of the run
            if (m & ~old) atomicAnd(v.words + ww, ~(m & ~old));
            break;
        }
    }
    if (ww > b) return true;
    for (uint32_t k = a; k < ww; ++k) atomicAnd(v.words + k, ~span_mask(p0, n, k));   // roll back
    return false;
}

// Random jumps until a run of n free pages is claimed (steps = jumps).  For
// n <= 32 the walk is pipelined: the LCG fixes every jump's words in
// advance, so the next kSpanAhead jumps' two words are in flight while a
// jump is judged and claimed, and the same words are examined in the same
// order.  Measured on the malloc workload (GB300): 1.64 G ops/s one jump
// ahead, 1.46 two ahead, 1.41 three ahead, 1.36 unpipelined.
constexpr int kSpanAhead = 1;
__device__ __forceinline__ int32_t walk_span(const PoolView& v, uint32_t n, int32_t seed0,
                                             uint32_t max_steps, int32_t* steps_out) {
    const uint32_t L = v.n_words32;
    int32_t x = seed0 & 0x7fffffff;   // walks run on 31-bit states
    uint32_t s = 0;
    if (n <= 32u && max_steps > 0u) {
        // ring of the next kSpanAhead jumps' words, loads in flight
        uint32_t pw[kSpanAhead], p0[kSpanAhead], p1[kSpanAhead];
#pragma unroll
        for (int k = 0; k < kSpanAhead; ++k) {
            x = lcg31(x);
            pw[k] = idx_hi(x, L);
            p0[k] = (uint32_t)k < max_steps ? load_word(v.words + pw[k]) : kFull32;
            p1[k] = (uint32_t)k < max_steps && pw[k] + 1u < L ? load_word(v.words + pw[k] + 1u) : kFull32;
        }
        while (s < max_steps) {
            const uint32_t w = pw[0], v0 = p0[0], v1 = p1[0];
            ++s;
#pragma unroll
            for (int k = 0; k + 1 < kSpanAhead; ++k) {
                pw[k] = pw[k + 1];
                p0[k] = p0[k + 1];
                p1[k] = p1[k + 1];
            }
            x = lcg31(x);                                  // jump s + kSpanAhead
            pw[kSpanAhead - 1] = idx_hi(x, L);
            const bool more = s + (uint32_t)kSpanAhead <= max_steps;
            p0[kSpanAhead - 1] = more ? load_word(v.words + pw[kSpanAhead - 1]) : kFull32;
            p1[kSpanAhead - 1] = more && pw[kSpanAhead - 1] + 1u < L ? load_word(v.words + pw[kSpanAhead - 1] + 1u)
                                                                     : kFull32;
            const int32_t found = span_in_pair(w, v0, v1, n, L);
            if (found >= 0 && claim_span(v, (uint32_t)found, n)) {
                if (steps_out) *steps_out = (int32_t)s;
                return found;
            }
        }
        if (steps_out) *steps_out = (int32_t)s;
        return -1;
    }
    while (s < max_steps) {
        ++s;
        x = lcg31(x);
        const int32_t found = find_span(v, idx_hi(x, L), n);
        if (found < 0) continue;
        if (claim_span(v, (uint32_t)found, n)) {
            if (steps_out) *steps_out = (int32_t)s;
            return found;
        }
    }
    if (steps_out) *steps_out = (int32_t)s;
    return -1;
}

// Affine jump-ahead of the LCG by lane + 1 steps: lcg31 applied lane + 1
// times to x is (aj * x + cj) mod 2^31.  The same table serves every walk of
// the warp, so it is computed once per call.
__device__ __forceinline__ void lcg_jump_for_lane(uint32_t lane, uint32_t& aj, uint32_t& cj) {
    aj = 1103515245u;
    cj = 12345u;
    for (uint32_t k = 0; k < lane; ++k) {
        cj = 1103515245u * cj + 12345u;
        aj *= 1103515245u;
    }
}

// Runs of need_n <= 32 pages (0 = none) for the lanes of a whole warp, each
// lane on its own LCG sequence from seed0; steps = jumps.  Every needing
// lane first takes one jump of its own (all in parallel).  Each lane still
// unserved is then walked by the whole warp, 32 of its jumps at a time:
// lane j judges the lane's jump s + j + 1 (its LCG state advanced j + 1
// steps at once) and the runs found are claimed in jump order.  In a run
// without races a lane gets the page the one-lane walk would give it, after
// the same jumps; a walk that keeps missing costs max_steps / 32 rounds
// instead of max_steps jumps.  The whole warp calls converged.
__device__ __forceinline__ int32_t walk_span_warp(const PoolView& v, uint32_t need_n, int32_t seed0,
                                                  uint32_t max_steps, int32_t* steps_out) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t L = v.n_words32;
    int32_t x = seed0 & 0x7fffffff;   // walks run on 31-bit states
    uint32_t s = 0;
    int32_t id = -1;
    if (need_n > 0u && max_steps > 0u) {
        s = 1;
        x = lcg31(x);
        const uint32_t w = idx_hi(x, L);
        const uint32_t v0 = load_word(v.words + w);
        const uint32_t v1 = w + 1u < L ? load_word(v.words + w + 1u) : kFull32;
        const int32_t f = span_in_pair(w, v0, v1, need_n, L);
        if (f >= 0 && claim_span(v, (uint32_t)f, need_n)) id = f;
    }
    uint32_t pend = __ballot_sync(kFull32, need_n > 0u && id < 0 && s < max_steps);
    uint32_t aj = 0u, cj = 0u;                             // jump ahead by lane + 1 steps
    if (pend) lcg_jump_for_lane(lane, aj, cj);
    while (pend) {
        const int l0 = __ffs((int)pend) - 1;
        const uint32_t x0 = (uint32_t)__shfl_sync(kFull32, x, l0);
        const uint32_t n0 = __shfl_sync(kFull32, need_n, l0);
        const uint32_t s0 = __shfl_sync(kFull32, s, l0);
        const int32_t xj = (int32_t)((aj * x0 + cj) & 0x7fffffffu);
        const uint32_t wj = idx_hi(xj, L);
        int32_t fj = -1;
        if (s0 + lane + 1u <= max_steps) {
            const uint32_t a0 = load_word(v.words + wj);
            const uint32_t a1 = wj + 1u < L ? load_word(v.words + wj + 1u) : kFull32;
            fj = span_in_pair(wj, a0, a1, n0, L);
        }
        uint32_t cm = __ballot_sync(kFull32, fj >= 0);
        int32_t got = -1;
        uint32_t used = 32u;
        while (cm) {                                       // claims in jump order
            const int j = __ffs((int)cm) - 1;
            cm &= cm - 1u;
            bool ok = false;
            if ((int)lane == j) ok = claim_span(v, (uint32_t)fj, n0);
            if (__shfl_sync(kFull32, ok, j)) {
                got = __shfl_sync(kFull32, fj, j);
                used = (uint32_t)j + 1u;
                break;
            }
        }
        const int32_t x_last = __shfl_sync(kFull32, xj, 31);   // the state 32 jumps on
        if ((int)lane == l0) {
            if (got >= 0) {
                id = got;
                s = s0 + used;
            } else {
                s = s0 + 32u < max_steps ? s0 + 32u : max_steps;
                x = x_last;
            }
        }
        pend = __ballot_sync(kFull32, need_n > 0u && id < 0 && s < max_steps);
    }
    if (steps_out) *steps_out = (int32_t)s;
    return id;
}

// ---------------------------------------------------------------------------
// FIFO free list (linked-list strategy, parallelPage.cu:342-440, restated
// lock-free).  get: reserve one free page on `avail`, take a head ticket,
// exchange the ring slot with -1 (bounded wait for the put that holds the
// ticket); put: take a tail ticket, CAS the id into the empty slot (bounded
// wait).  A wait that runs out records a timeout and returns -1 / false.
// The bitmap is kept in step so occupancy and invariants read the same.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int32_t fifo_get(const PoolView& v, FifoState* st, int32_t* ring,
                                            DevStats* stats, int32_t* spins) {
    unsigned long long old = atomicAdd(&st->avail, ~0ull);   // avail -= 1
    if ((long long)old <= 0) {
        atomicAdd(&st->avail, 1ull);
        if (spins) *spins = 0;
        return -1;
    }
    unsigned long long t = atomicAdd(&st->head, 1ull);
    int32_t* slot = ring + (t % v.n_pages);
    uint32_t k = 0;
    int32_t id = atomicExch(slot, -1);
    while (id < 0 && k < kFifoSpinLimit) {
        __nanosleep(64);
        ++k;
        id = atomicExch(slot, -1);
    }
    if (spins) *spins = (int32_t)k + 1;
    if (id < 0) {
        atomicAdd(&stats->timeouts, 1ull);
        return -1;
    }
    atomicOr(v.words + ((uint32_t)id >> 5), 1u << ((uint32_t)id & 31u));
    return id;
}

__device__ __forceinline__ bool fifo_put(const PoolView& v, FifoState* st, int32_t* ring,
                                         DevStats* stats, int32_t id) {
    atomicAnd(v.words + ((uint32_t)id >> 5), ~(1u << ((uint32_t)id & 31u)));
    unsigned long long t = atomicAdd(&st->tail, 1ull);
    int32_t* slot = ring + (t % v.n_pages);
    uint32_t k = 0;
    while (atomicCAS(slot, -1, id) != -1) {
        if (++k >= kFifoSpinLimit) {
            atomicAdd(&stats->timeouts, 1ull);
            return false;
        }
        __nanosleep(64);
    }
    atomicAdd(&st->avail, 1ull);
    return true;
}

// ---------------------------------------------------------------------------
// Frees.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void free_page(const PoolView& v, int32_t id) {
    atomicAnd(v.words + ((uint32_t)id >> 5), ~(1u << ((uint32_t)id & 31u)));
}

__device__ __forceinline__ void free_run(const PoolView& v, int32_t id, uint32_t n) {
    uint32_t st = (uint32_t)id & 31u;
    uint32_t m = (n >= 32u ? kFull32 : ((1u << n) - 1u)) << st;
    atomicAnd(v.words + ((uint32_t)id >> 5), ~m);
}

// Warp-aggregated free: lanes freeing pages of the same word merge their
// bits (__match_any_sync + __reduce_or_sync) and one lane issues the AND.
// `active` = lanes calling converged; lanes with id < 0 free nothing.
__device__ __forceinline__ void free_page_warp(const PoolView& v, uint32_t active, int32_t id) {
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t w = id >= 0 ? ((uint32_t)id >> 5) : 0xffffffffu;
    uint32_t bit = id >= 0 ? (1u << ((uint32_t)id & 31u)) : 0u;
    uint32_t peers = __match_any_sync(active, w);
    uint32_t merged = __reduce_or_sync(peers, bit);
    if (id >= 0 && (__ffs((int)peers) - 1) == (int)lane) atomicAnd(v.words + w, ~merged);
}

// ---------------------------------------------------------------------------
// Launch budget: fail fast in an exhausted pool.  A pass over the bitmap just
// before the launch counts the free pages F.  Request r of the launch may
// take a page only if r < F: the requests past the pages that were free
// fail at once instead of walking to their step bound, and no more pages are
// granted than were free at the start -- with no atomic at all, so the
// launch never contends on a shared counter.  When the launch asks for at
// least half of the F free pages (`list_mode`), the pass also lists the free
// pages in ascending order, and request r takes list[r] directly instead of
// searching for it.  A null budget grants every request.
// ---------------------------------------------------------------------------
struct LaunchBudget {
    long long free_at_start;    // F
    int32_t list_mode;          // 1: list[0..F) holds the free pages in order
    int32_t pad;
};

__device__ __forceinline__ bool budget_grants(const LaunchBudget* b, unsigned long long r) {
    return !b || (long long)r < __ldcg(&b->free_at_start);
}

// A listed page, claimed with one atomicOr; -1 if another claim (a launch on
// another stream) took it first.
__device__ __forceinline__ int32_t take_listed(const PoolView& v, const int32_t* list, long long index) {
    const int32_t p = __ldcg(list + index);
    const uint32_t bit = 1u << ((uint32_t)p & 31u);
    return (atomicOr(v.words + ((uint32_t)p >> 5), bit) & bit) ? -1 : p;
}

__device__ __forceinline__ void* page_address(const PoolView& v, int32_t id) {
    return (void*)(v.base + (size_t)(uint32_t)id * v.page_size);
}

__device__ __forceinline__ int32_t page_id(const PoolView& v, const void* p) {
    size_t off = (size_t)((const char*)p - v.base);
    if ((const char*)p < v.base || off >= (size_t)v.n_pages * v.page_size) return -1;
    return (int32_t)(off / v.page_size);
}

#endif  // __CUDACC__
}  // namespace pbm
