// cpu_replay.cpp -- std::atomic host replay of the reference's bitmap random
// walks (the CPU baseline; TEST INFRASTRUCTURE / CPU BASELINE ONLY).
//
// Restates, on host threads, the per-thread walks of
//   source/RandomWalkBasic_BM.cuh:60-102  (word probe: random word, claim its
//                                          first clear bit with an atomic OR)
//   source/RandomWalkBasic.cuh:54-84      (page probe, here on the bitmap)
// with the reference LCG (source/RNG_LCG.cuh:9-12) and the same bitmap layout
// as the GPU pool, applied to the alloc+free churn workload: request i
// claims a new page, frees the page held in its slot and stores the new one.
// Word updates use GCC __atomic builtins (fetch_or / fetch_and), which are
// std::atomic operations on plain storage and build on x86-64 and aarch64.
#include <atomic>
#include <chrono>
#include <cstdint>
#include <thread>
#include <vector>

#include "pbm_oracle.h"

namespace {

inline uint32_t idx_hi(int32_t x, uint32_t n) {
    return (uint32_t)((((uint64_t)((uint32_t)x & 0x7fffffffu)) * (uint64_t)n) >> 31);
}

inline int32_t walk_word(uint32_t* words, uint32_t L, int32_t x, uint32_t max_steps, uint32_t* steps) {
    uint32_t s = 0;
    while (s < max_steps) {
        ++s;
        x = orc_lcg(x);
        uint32_t w = idx_hi(x, L);
        uint32_t v = __atomic_load_n(words + w, __ATOMIC_RELAXED);
        while (v != 0xffffffffu) {
            int b = __builtin_ctz(~v);
            uint32_t bit = 1u << b;
            uint32_t old = __atomic_fetch_or(words + w, bit, __ATOMIC_RELAXED);
            if (!(old & bit)) { *steps = s; return (int32_t)(w * 32u + (uint32_t)b); }
            v = old | bit;
        }
    }
    *steps = s;
    return -1;
}

inline int32_t walk_page(uint32_t* words, uint32_t T, int32_t x, uint32_t max_steps, uint32_t* steps) {
    uint32_t s = 0;
    while (s < max_steps) {
        ++s;
        x = orc_lcg(x);
        uint32_t p = idx_hi(x, T);
        uint32_t* wp = words + (p >> 5);
        uint32_t bit = 1u << (p & 31u);
        if (__atomic_load_n(wp, __ATOMIC_RELAXED) & bit) continue;
        if (!(__atomic_fetch_or(wp, bit, __ATOMIC_RELAXED) & bit)) { *steps = s; return (int32_t)p; }
    }
    *steps = s;
    return -1;
}

}  // namespace

extern "C" {

// Churn: n_pairs alloc+free pairs over `threads` host threads.  Thread t owns
// the held slots [t*H/threads, (t+1)*H/threads) and walks them cyclically.
// walk: 0 = page probe, 1 = word probe.  Returns wall seconds of the
// parallel region; ok/fail/steps are totals.
double orc_cpu_churn(uint32_t* words, uint64_t n_pages, int32_t* held, uint64_t n_held, uint64_t n_pairs,
                     uint32_t seed, int threads, int walk, uint32_t max_steps, uint64_t* ok, uint64_t* fail,
                     uint64_t* steps) {
    if (threads < 1) threads = 1;
    const uint32_t T = (uint32_t)n_pages;
    const uint32_t L = (uint32_t)((n_pages + 31u) / 32u);
    std::vector<uint64_t> oks(threads), fails(threads), stps(threads);
    std::atomic<int> ready{0};
    std::atomic<bool> go{false};
    auto body = [&](int t) {
        const uint64_t lo = n_held * (uint64_t)t / (uint64_t)threads;
        const uint64_t hi = n_held * (uint64_t)(t + 1) / (uint64_t)threads;
        const uint64_t span = hi - lo;
        const uint64_t mine = n_pairs * (uint64_t)(t + 1) / (uint64_t)threads - n_pairs * (uint64_t)t / (uint64_t)threads;
        const uint64_t q0 = n_pairs * (uint64_t)t / (uint64_t)threads;
        uint64_t o = 0, f = 0, st = 0;
        ready.fetch_add(1);
        while (!go.load(std::memory_order_acquire)) {}
        for (uint64_t i = 0; i < mine; ++i) {
            uint32_t s = 0;
            int32_t x0 = orc_seed(seed, (uint32_t)(q0 + i));
            int32_t id = walk ? walk_word(words, L, x0, max_steps, &s) : walk_page(words, T, x0, max_steps, &s);
            st += s;
            if (id < 0) { ++f; continue; }
            ++o;
            if (span) {
                uint64_t slot = lo + (i % span);
                int32_t old = held[slot];
                held[slot] = id;
                if (old >= 0)
                    __atomic_fetch_and(words + ((uint32_t)old >> 5), ~(1u << ((uint32_t)old & 31u)), __ATOMIC_RELAXED);
            }
        }
        oks[t] = o; fails[t] = f; stps[t] = st;
    };
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) pool.emplace_back(body, t);
    while (ready.load() < threads) {}
    auto t0 = std::chrono::steady_clock::now();
    go.store(true, std::memory_order_release);
    for (auto& th : pool) th.join();
    auto t1 = std::chrono::steady_clock::now();
    uint64_t O = 0, F = 0, S = 0;
    for (int t = 0; t < threads; ++t) { O += oks[t]; F += fails[t]; S += stps[t]; }
    if (ok) *ok = O;
    if (fail) *fail = F;
    if (steps) *steps = S;
    return std::chrono::duration<double>(t1 - t0).count();
}

// Claim, write, free (the 64-byte-page workload, unitTest1.5.cu:127-150 with
// getPagePtr payloads): request i claims a page with the page-probe walk,
// writes i into the first payload_bytes of the page and frees it at once;
// `reps` passes over the n requests, split evenly over `threads` host threads.
// Returns wall seconds of the parallel region; ok/steps are totals.
double orc_cpu_claim_write_free(uint32_t* words, uint64_t n_pages, uint8_t* pages, uint32_t page_size,
                                uint32_t payload_bytes, uint64_t n, uint32_t seed, int threads, uint32_t reps,
                                uint32_t max_steps, uint64_t* ok, uint64_t* steps) {
    if (threads < 1) threads = 1;
    const uint32_t T = (uint32_t)n_pages;
    const uint32_t words_per = payload_bytes / 4u;
    std::vector<uint64_t> oks(threads), stps(threads);
    std::atomic<int> ready{0};
    std::atomic<bool> go{false};
    auto body = [&](int t) {
        const uint64_t lo = n * (uint64_t)t / (uint64_t)threads;
        const uint64_t hi = n * (uint64_t)(t + 1) / (uint64_t)threads;
        uint64_t o = 0, st = 0;
        ready.fetch_add(1);
        while (!go.load(std::memory_order_acquire)) {}
        for (uint32_t r = 0; r < reps; ++r) {
            for (uint64_t i = lo; i < hi; ++i) {
                uint32_t s = 0;
                const int32_t id = walk_page(words, T, orc_seed(seed, (uint32_t)i), max_steps, &s);
                st += s;
                if (id < 0) continue;
                ++o;
                int32_t* pg = reinterpret_cast<int32_t*>(pages + (uint64_t)(uint32_t)id * page_size);
                for (uint32_t k = 0; k < words_per; ++k) __atomic_store_n(pg + k, (int32_t)i, __ATOMIC_RELAXED);
                __atomic_fetch_and(words + ((uint32_t)id >> 5), ~(1u << ((uint32_t)id & 31u)), __ATOMIC_RELEASE);
            }
        }
        oks[t] = o;
        stps[t] = st;
    };
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) pool.emplace_back(body, t);
    while (ready.load() < threads) {}
    auto t0 = std::chrono::steady_clock::now();
    go.store(true, std::memory_order_release);
    for (auto& th : pool) th.join();
    auto t1 = std::chrono::steady_clock::now();
    uint64_t O = 0, S = 0;
    for (int t = 0; t < threads; ++t) { O += oks[t]; S += stps[t]; }
    if (ok) *ok = O;
    if (steps) *steps = S;
    return std::chrono::duration<double>(t1 - t0).count();
}

int orc_hw_threads(void) {
    unsigned n = std::thread::hardware_concurrency();
    return n ? (int)n : 1;
}

}  // extern "C"
