// bufmgr.cu -- buffer manager with CLOCK (second-chance) replacement.
//
// The reference has page allocators only; its SingleClock / DistClock arms
// sweep the free map (parallelPage.cu:491-509, 571-592) but there is no page
// table, no reference bits and no eviction.  This file defines the buffer
// manager on those sweep mechanics.  Its state, laid out so that a hit
// touches one 32-byte sector:
//
//   pt[p]          one 64-bit word per logical page: the frame holding p in
//                  the high 32 bits (-1 not resident, -2 being loaded, -3 a
//                  load that failed and is being left), the CLOCK reference
//                  bit in bit 31, a guard bit (bit 30, always set between
//                  operations) and the page's pins in bits 0..29.  The guard
//                  lets a release subtract its pins first and check after:
//                  a release of more pins than the page holds borrows from
//                  the guard instead of the reference bit or the frame, and
//                  is added back
//   frame_page[f]  the page frame f holds (0xffffffff: empty)
//   hands          SINGLE: one shared hand (atomicAdd); DIST: per-slot hands,
//                  each starting at its own frame and advancing privately
//
// fetch(p) for k requests of p (the lanes of a warp that fetch one page
// merge into one atomic): add k pins to pt[p] with one atomicAdd.  Resident
// -> a hit; the reference bit is set with a second atomic only if it was
// clear.  Not resident and no pins before -> this request loads the page:
// it marks the entry loading, sweeps -- frames whose page is pinned are
// passed, referenced ones lose their bit (second chance), the first
// unpinned unreferenced frame is taken by a compare-and-swap of its page's
// entry to not-resident (eviction) -- optionally copies the page from the
// backing store, and publishes the frame (one miss; its k-1 companions are
// hits).  Otherwise another request is loading it: the pins are already
// counted, so the request waits (bounded) for the frame.  A load that finds
// no frame within max_sweep hand steps fails all its k requests; requests
// waiting on it leave (the last one out clears the failure) and try again,
// where a second failure is final.  Releases unpin through frame_page.
// One thread running the rounds in order reproduces the single-thread
// replay of these semantics exactly.
#include <cstring>
#include <new>

#include "internal.cuh"

namespace pbm {
namespace {

constexpr uint32_t kEmptyPage = 0xffffffffu;
constexpr int32_t kNotResident = -1;
constexpr int32_t kLoading = -2;
constexpr int32_t kFailed = -3;
constexpr unsigned long long kFrameUnit = 1ull << 32;
constexpr unsigned long long kRef = 1ull << 31;
constexpr uint32_t kGuard = 1u << 30;
constexpr uint32_t kPinField = 0x7fffffffu;   // guard + pins
constexpr unsigned long long kEntryNotResident = ((unsigned long long)(uint32_t)kNotResident << 32) | kGuard;
constexpr unsigned long long kEntryFailed = ((unsigned long long)(uint32_t)kFailed << 32) | kGuard;
constexpr uint32_t kFetchSpinLimit = 1u << 16;   // polls of a page another request is loading
constexpr uint32_t kFetchAttempts = 1024u;        // fetches retried after a failed load

__device__ __forceinline__ int32_t e_frame(unsigned long long e) { return (int32_t)(e >> 32); }
// Pins of an entry; while another release's over-subtraction has borrowed
// the guard, this reads as a huge count (the page counts as pinned).
__device__ __forceinline__ uint32_t e_pins(unsigned long long e) { return ((uint32_t)e & kPinField) - kGuard; }
__device__ __forceinline__ bool e_ref(unsigned long long e) { return (e & kRef) != 0ull; }

struct BmStats {
    unsigned long long hits, misses, evictions, failures, unpins, bad_unpins, timeouts, pad;
};

struct BmView {
    unsigned long long* pt;  // n_logical entries
    uint32_t* frame_page;    // n_frames
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

struct BmAcc {
    unsigned long long hits = 0, misses = 0, evictions = 0, failures = 0, timeouts = 0;
};

// Frame f as a victim for `page`: empty frames are taken by writing their
// page; a mapped frame is taken by turning its page's entry from (f, no
// reference, no pins) to not resident.  `e` is the entry read for frame f's
// page q (unused for empty frames).  Returns true if this thread took f.
__device__ __forceinline__ bool take_frame(const BmView& b, uint32_t f, uint32_t q, unsigned long long e,
                                           uint32_t page, uint32_t* old_page) {
    if (q == kEmptyPage) {
        if (atomicCAS(b.frame_page + f, kEmptyPage, page) != kEmptyPage) return false;
        *old_page = kEmptyPage;
        return true;
    }
    if (atomicCAS(b.pt + q, e, kEntryNotResident) != e) return false;
    b.frame_page[f] = page;
    *old_page = q;
    return true;
}

// One frame under the hand: 0 pass, 1 candidate (q, e filled in).  A
// referenced frame loses its reference bit here (second chance).
// judge: the same for frame f holding page q whose entry e was read.
__device__ __forceinline__ bool judge(const BmView& b, uint32_t f, uint32_t q, unsigned long long e) {
    if (q == kEmptyPage) return true;
    if (q >= b.n_logical) return false;
    if (e_frame(e) != (int32_t)f || e_pins(e) != 0u) return false;   // pinned, or changing hands
    if (e_ref(e)) {
        atomicAnd(b.pt + q, ~kRef);
        return false;
    }
    return true;
}

__device__ __forceinline__ int examine(const BmView& b, uint32_t f, uint32_t* q_out, unsigned long long* e_out) {
    const uint32_t q = __ldcg(b.frame_page + f);
    *q_out = q;
    const unsigned long long e = (q < b.n_logical) ? __ldcg(b.pt + q) : 0ull;
    *e_out = e;
    return judge(b, f, q, e) ? 1 : 0;
}

// Per-slot hand (DistClock, parallelPage.cu:571-592): the slot's hand is
// private, so it reads the next kLookahead frames' pages in one round trip
// and then examines them in hand order exactly as the one-step sweep does,
// stopping at the victim (the hand ends just past it, and frames beyond it
// are untouched).  Never more frames at once than the pool has, so one
// batch never sees a frame twice.
constexpr uint32_t kLookahead = 8;

__device__ __forceinline__ int32_t sweep_private(const BmView& b, uint32_t page, uint32_t slot,
                                                 uint32_t* old_page) {
    uint32_t arm = b.arms[slot];
    if (arm >= b.n_frames) arm %= b.n_frames;
    const uint32_t width = b.n_frames < kLookahead ? b.n_frames : kLookahead;
    int32_t out = -1;
    for (uint32_t done = 0; done < b.max_sweep && out < 0;) {
        uint32_t qs[kLookahead];
#pragma unroll
        for (uint32_t j = 0; j < kLookahead; ++j) {
            if (j < width) {
                uint32_t f = arm + j;
                if (f >= b.n_frames) f -= b.n_frames;
                qs[j] = __ldcg(b.frame_page + f);
            }
        }
        unsigned long long es[kLookahead];
#pragma unroll
        for (uint32_t j = 0; j < kLookahead; ++j)
            es[j] = (j < width && qs[j] < b.n_logical) ? __ldcg(b.pt + qs[j]) : 0ull;
#pragma unroll
        for (uint32_t j = 0; j < kLookahead; ++j) {
            if (j >= width || done >= b.max_sweep || out >= 0) break;
            const uint32_t f = arm;
            arm = f + 1u == b.n_frames ? 0u : f + 1u;
            ++done;
            const uint32_t q = qs[j];
            const unsigned long long e = es[j];
            if (q != kEmptyPage) {
                if (q >= b.n_logical || e_frame(e) != (int32_t)f || e_pins(e) != 0u) continue;
                if (e_ref(e)) { atomicAnd(b.pt + q, ~kRef); continue; }   // second chance
            }
            if (take_frame(b, f, q, e, page, old_page)) out = (int32_t)f;
        }
    }
    b.arms[slot] = arm;
    return out;
}

// Victim search of one thread; returns a frame now holding `page` (the
// entry of `page` itself is published by the caller) and its old page.  The
// shared hand advances one position per atomic (parallelPage.cu:491-509).
template <bool DIST>
__device__ __forceinline__ int32_t sweep(const BmView& b, uint32_t page, uint32_t slot, uint32_t* old_page) {
    if constexpr (DIST) return sweep_private(b, page, slot, old_page);
    for (uint32_t i = 0; i < b.max_sweep; ++i) {
        const uint32_t f = (uint32_t)(atomicAdd(b.single_hand, 1ull) % b.n_frames);
        uint32_t q;
        unsigned long long e = 0;
        if (examine(b, f, &q, &e) && take_frame(b, f, q, e, page, old_page)) return (int32_t)f;
    }
    return -1;
}

__device__ __forceinline__ void copy_frame(const BmView& b, uint32_t page, int32_t h) {
    const int4* src = reinterpret_cast<const int4*>(b.backing + (size_t)page * b.frame_size);
    int4* dst = reinterpret_cast<int4*>(b.frames + (size_t)h * b.frame_size);
    for (uint32_t k = 0; k < b.frame_size / 16u; ++k) dst[k] = src[k];
}

// Takes k pins of `page` off its entry; the last request to leave a failed
// load clears the failure.
__device__ __forceinline__ void leave(const BmView& b, uint32_t page, uint32_t k) {
    const unsigned long long old = atomicAdd(b.pt + page, 0ull - (unsigned long long)k);
    if (e_frame(old) == kFailed && e_pins(old) == k) atomicCAS(b.pt + page, kEntryFailed, kEntryNotResident);
}

// The loader's end of a load: publish frame h (entry loading -> h, reference
// bit set) or, when no frame was found, mark the load failed and take the
// loader's own k pins off.
__device__ __forceinline__ void publish(const BmView& b, uint32_t page, int32_t h, uint32_t old_page, uint32_t k,
                                        BmAcc& acc) {
    if (h >= 0) {
        if (old_page != kEmptyPage) ++acc.evictions;
        // the frame's bytes before the entry that names the frame.  Without a
        // copy nothing needs the order: a sweep that reads frame_page[h]
        // before the entry is published, or the old page's entry after the
        // eviction, finds an entry that does not name h and passes the frame
        if (b.frames && b.backing) __threadfence();
        atomicAdd(b.pt + page, (unsigned long long)(h - kLoading) * kFrameUnit + kRef);
        acc.misses += 1u;
        acc.hits += k - 1u;
    } else {
        const unsigned long long old = atomicAdd(b.pt + page, (0ull - kFrameUnit) - (unsigned long long)k);
        if (e_pins(old) == k) atomicCAS(b.pt + page, kEntryFailed, kEntryNotResident);
        acc.failures += k;
    }
}

enum : int { kStHit = 1, kStLoad = 2, kStWait = 3 };

// The state of a fetch whose k pins were just added (`old`: the entry before
// the add): a hit (reference bit set if it was clear), the load of
// a page not resident and unpinned (entry marked loading), or a wait for
// another request's load.
__device__ __forceinline__ int fetch_state(const BmView& b, uint32_t page, unsigned long long old, int32_t* frame) {
    const int32_t f = e_frame(old);
    if (f >= 0) {
        if (!e_ref(old)) atomicOr(b.pt + page, kRef);
        *frame = f;
        return kStHit;
    }
    if (f == kNotResident && e_pins(old) == 0u) {
        atomicAdd(b.pt + page, 0ull - kFrameUnit);   // not resident -> loading
        return kStLoad;
    }
    return kStWait;
}

// The first step of a fetch of `page` for k requests: add their pins.
// Returns the state and, for a hit, the frame.
__device__ __forceinline__ int begin_fetch(const BmView& b, uint32_t page, uint32_t k, int32_t* frame) {
    return fetch_state(b, page, atomicAdd(b.pt + page, (unsigned long long)k), frame);
}

// A request whose pins are registered on a page another request is loading:
// wait (bounded) for the frame.  Returns the frame, kFailed if that load
// failed, or kLoading if the wait ran out.
__device__ __forceinline__ int32_t wait_loaded(const BmView& b, uint32_t page) {
    for (uint32_t i = 0; i < kFetchSpinLimit; ++i) {
        const int32_t f = e_frame(__ldcg(b.pt + page));
        if (f >= 0 || f == kFailed) return f;
        __nanosleep(32);
    }
    return kLoading;
}

// A whole fetch of `page` for k requests by one thread (the single-thread
// replay, and the per-slot-hand policy).
template <bool DIST>
__device__ __forceinline__ int32_t fetch_k(const BmView& b, uint32_t page, uint32_t slot, uint32_t k, BmAcc& acc) {
    for (uint32_t attempt = 0; attempt < kFetchAttempts; ++attempt) {
        int32_t f = -1;
        const int st = begin_fetch(b, page, k, &f);
        if (st == kStHit) {
            acc.hits += k;
            return f;
        }
        if (st == kStLoad) {
            uint32_t old_page = kEmptyPage;
            const int32_t h = sweep<DIST>(b, page, slot, &old_page);
            if (h >= 0 && b.backing && b.frames) copy_frame(b, page, h);
            publish(b, page, h, old_page, k, acc);
            return h;
        }
        f = wait_loaded(b, page);
        if (f >= 0) {
            acc.hits += k;
            return f;
        }
        leave(b, page, k);
        if (f == kLoading) {
            acc.timeouts += k;
            return -1;
        }
        __nanosleep(64);   // the failed load is being left: try again
    }
    acc.timeouts += k;
    return -1;
}

// Warp-cooperative CLOCK sweep on the single hand.  The lanes in `loaders`
// (each the loader of its own `page`, its entry already marked loading) need
// victim frames.  Per window the warp takes 32 consecutive hand positions
// with one atomicAdd and every lane examines one frame, as the one-thread
// sweep does.  Candidates go in hand order to the loaders in lane order,
// each taken with the one-thread sweep's compare-and-swap (a pin that
// arrived in between makes it fail and the loader waits for the next
// window); candidates beyond the loaders' need are passed.  A loader gives
// up after its max_sweep positions.  The whole warp calls converged.
struct SweepWin {
    uint32_t f, q;           // this lane's frame and the page it held
    unsigned long long e;    // that page's entry as read
    bool cand;
};

__device__ __forceinline__ SweepWin sweep_window(const BmView& b) {
    unsigned long long base = 0;
    if ((threadIdx.x & 31u) == 0u) base = atomicAdd(b.single_hand, 32ull);
    base = __shfl_sync(0xffffffffu, base, 0);
    SweepWin w;
    w.f = (uint32_t)((base + (threadIdx.x & 31u)) % b.n_frames);
    w.cand = examine(b, w.f, &w.q, &w.e) != 0;
    return w;
}

// Hands one window's candidates to the loaders; returns the loaders still
// without a frame.  *out / *old_page: the lane's frame and the page it held.
__device__ __forceinline__ uint32_t sweep_assign(const BmView& b, const SweepWin& w, uint32_t loaders,
                                                 uint32_t page, int32_t* out, uint32_t* old_page) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t lt = (1u << lane) - 1u;
    const uint32_t cm = __ballot_sync(0xffffffffu, w.cand);
    const int n_load = __popc(loaders);
    // candidate of rank k serves the loader of rank k
    const int k = __popc(cm & lt);
    const int target = (w.cand && k < n_load) ? (int)nth_set_bit(loaders, k) : -1;
    const uint32_t tpage = __shfl_sync(0xffffffffu, page, target < 0 ? (int)lane : target);
    uint32_t victim_old = kEmptyPage;
    const bool took = target >= 0 && take_frame(b, w.f, w.q, w.e, tpage, &victim_old);
    const uint32_t tm = __ballot_sync(0xffffffffu, took);
    const bool is_loader = (loaders >> lane) & 1u;
    const int r = __popc(loaders & lt);
    const int src = (is_loader && r < __popc(cm)) ? (int)nth_set_bit(cm, r) : -1;
    const uint32_t got_f = __shfl_sync(0xffffffffu, w.f, src < 0 ? (int)lane : src);
    const uint32_t got_old = __shfl_sync(0xffffffffu, victim_old, src < 0 ? (int)lane : src);
    if (src >= 0 && ((tm >> src) & 1u)) {
        *out = (int32_t)got_f;
        *old_page = got_old;
    }
    return __ballot_sync(0xffffffffu, is_loader && *out < 0);
}

// The whole sweep: `first`, if given, is a window the warp already took and
// examined (it counts against max_sweep).  Returns the lane's frame (-1 if
// none) and the page it held.
__device__ __forceinline__ int32_t sweep_warp(const BmView& b, uint32_t loaders, uint32_t page, uint32_t* old_page,
                                              const SweepWin* first = nullptr) {
    int32_t out = -1;
    const uint32_t max_windows = b.max_sweep > 32u ? (b.max_sweep + 31u) / 32u : 1u;
    uint32_t it = 0;
    if (first) {
        loaders = sweep_assign(b, *first, loaders, page, &out, old_page);
        it = 1;
    }
    for (; loaders != 0u && it < max_windows; ++it) {
        const SweepWin w = sweep_window(b);
        loaders = sweep_assign(b, w, loaders, page, &out, old_page);
    }
    return out;
}

// The loaders' side of a cooperative miss: copy the new pages from the
// backing store with the whole warp, then publish the entries.  The warp's
// copies are one flat run of 16-byte pieces (loader by loader, piece by
// piece); each lane has kCopyInFlight of its pieces loading at once before
// it stores them, so a warp keeps 32 x kCopyInFlight loads in flight across
// its loaders' pages.  The whole warp calls converged.
constexpr uint32_t kCopyInFlight = 4;

template <bool COPY>
__device__ __forceinline__ void finish_loads_warp(const BmView& b, bool loader, uint32_t page, int32_t h,
                                                  uint32_t old_page, uint32_t k, BmAcc& acc) {
    if (COPY) {
        const uint32_t lane = threadIdx.x & 31u;
        const uint32_t n16 = b.frame_size / 16u;
        const uint32_t todo = __ballot_sync(0xffffffffu, loader && h >= 0);
        const uint32_t total = (uint32_t)__popc(todo) * n16;
        for (uint32_t base = 0; base < total; base += 32u * kCopyInFlight) {
            int4 v[kCopyInFlight];
            int4* dst[kCopyInFlight];
#pragma unroll
            for (uint32_t u = 0; u < kCopyInFlight; ++u) {
                const uint32_t c = base + u * 32u + lane;
                const uint32_t li = (c < total ? c : 0u) / n16;
                const int l = (int)nth_set_bit(todo, (int)li);   // every lane shuffles
                const uint32_t pg = __shfl_sync(0xffffffffu, page, l);
                const int32_t fr = __shfl_sync(0xffffffffu, h, l);
                const uint32_t j = c - li * n16;
                dst[u] = nullptr;
                if (c < total) {
                    v[u] = reinterpret_cast<const int4*>(b.backing + (size_t)pg * b.frame_size)[j];
                    dst[u] = reinterpret_cast<int4*>(b.frames + (size_t)(uint32_t)fr * b.frame_size) + j;
                }
            }
#pragma unroll
            for (uint32_t u = 0; u < kCopyInFlight; ++u)
                if (dst[u]) *dst[u] = v[u];
        }
        __syncwarp();
    }
    if (loader) publish(b, page, h, old_page, k, acc);
}

// A release of k pins of `page` is one atomic: subtract first, then check
// that the page was resident -- in frame `frame` when the caller named the
// frame (frame < 0: any frame) -- and held at least k pins.  A release that
// was not is added back and counted bad; the guard bit keeps the borrowed
// pins away from the reference bit and the frame meanwhile.
__device__ __forceinline__ unsigned long long release_issue(const BmView& b, uint32_t page, uint32_t k) {
    return atomicAdd(b.pt + page, 0ull - (unsigned long long)k);
}

__device__ __forceinline__ void release_check(const BmView& b, uint32_t page, int32_t frame, uint32_t k,
                                              unsigned long long old, unsigned long long& ok,
                                              unsigned long long& bad) {
    const int32_t of = e_frame(old);
    if (of < 0 || (frame >= 0 && of != frame) || e_pins(old) < k) {
        atomicAdd(b.pt + page, (unsigned long long)k);
        bad += k;
        return;
    }
    ok += k;
}

// The page a release names: BYPAGE, the page itself (negative: nothing to
// release); else a frame, whose page frame_page names.  Returns false when
// there is nothing to release; out-of-range names are counted bad.
template <bool BYPAGE>
__device__ __forceinline__ bool release_target(const BmView& b, int32_t v, uint32_t k, uint32_t* page,
                                               int32_t* frame, unsigned long long& bad) {
    if (v < 0) return false;
    if constexpr (BYPAGE) {
        if ((uint32_t)v >= b.n_logical) { bad += k; return false; }
        *page = (uint32_t)v;
        *frame = -1;
    } else {
        if ((uint32_t)v >= b.n_frames) return false;
        const uint32_t q = __ldcg(b.frame_page + v);
        if (q >= b.n_logical) { bad += k; return false; }
        *page = q;
        *frame = v;
    }
    return true;
}

// Per-block merge tables (shared memory): the block's requests for one key
// meet in one slot, and one lane issues one atomic for all of them.  Under a
// skewed stream the hottest pages are in nearly every warp's requests, so
// merging within the block rather than the warp divides the atomics that
// queue on one page's entry by the block's warps.  Releases by page share
// the fetches' table: a block that releases and fetches one page moves its
// pins with one atomic.
constexpr uint32_t kMergeSlots = 1024;           // >= 2 x the keys of one block (256 fetches + 256 releases)
constexpr uint32_t kMergeEmpty = 0xffffffffu;   // no page or frame id reaches it
constexpr uint32_t kMergeFirst = 1u << 31;

struct MergeTables {
    uint32_t fkey[kMergeSlots];   // pages (and, releasing by page, released pages)
    uint32_t fcnt[kMergeSlots];   // fetches of the page
    uint32_t frel[kMergeSlots];   // releases of the page (releasing by page)
    int32_t fres[kMergeSlots];    // the fetch's frame
    uint32_t rkey[kMergeSlots];   // released frames (releasing by frame)
    uint32_t rcnt[kMergeSlots];
};

// Adds c to cnt[slot of key]; returns the slot, with kMergeFirst set for the
// lane whose add came first (the slot's leader for that count).  A table
// never holds more keys than half its slots, so a slot is found.
__device__ __forceinline__ uint32_t merge_insert(uint32_t* keys, uint32_t* cnt, uint32_t key, uint32_t c) {
    uint32_t h = (key * 2654435761u) >> 22;   // 10 bits: kMergeSlots
    for (uint32_t probe = 0; probe < kMergeSlots; ++probe) {
        const uint32_t prev = atomicCAS(keys + h, kMergeEmpty, key);
        if (prev == kMergeEmpty || prev == key) return atomicAdd(cnt + h, c) == 0u ? (h | kMergeFirst) : h;
        h = (h + 1u) & (kMergeSlots - 1u);
    }
    return kMergeEmpty;   // not reached
}

// The many-thread round.  Per block iteration every lane takes release i
// and fetch i (i = the block's base + threadIdx.x); lanes merge by key in the
// warp (match) and then in the block (the tables), and each key's leader
// issues its atomic: the fetch's pin (with the block's releases of the page,
// releasing by page), and other releases while the pins are in flight.  The
// fetch's result goes back through the table to every lane that asked for
// the page.  With the single hand each warp also takes and examines its
// first sweep window while its pins are in flight: nearly every warp has a
// miss, and one that has none has still moved the hand over 32 frames as a
// sweep does (clearing reference bits, evicting nothing).  Releases of one
// round may land after other blocks' fetches of the same round; a sweep
// that meets a page whose release has not landed yet passes it as pinned,
// as it would any pinned page.
template <bool DIST, bool BYPAGE, bool COPY>
__device__ __forceinline__ void round_blocks(const BmView& b, const int32_t* release_of, const int32_t* release_idx,
                                             uint32_t n_release, const int32_t* pages, uint32_t n, uint32_t slot0,
                                             int32_t* frames_out, int32_t* held_out, unsigned long long& ok,
                                             unsigned long long& bad, BmAcc& acc) {
    __shared__ MergeTables t;
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t work = n > n_release ? n : n_release;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    // block-uniform trip count
    for (uint64_t bbase = (uint64_t)blockIdx.x * blockDim.x; bbase < work; bbase += stride) {
        const uint64_t i = bbase + threadIdx.x;
        unsigned long long hbase = 0;
        if (!DIST && lane == 0u) hbase = atomicAdd(b.single_hand, 32ull);   // the first sweep window
        const int32_t ri = i < n_release ? __ldg(release_idx + i) : -1;
        const int32_t p = i < n ? __ldg(pages + i) : -1;
        for (uint32_t s = threadIdx.x; s < kMergeSlots; s += blockDim.x) {
            t.fkey[s] = kMergeEmpty;
            t.fcnt[s] = 0u;
            t.frel[s] = 0u;
            if (!BYPAGE) {
                t.rkey[s] = kMergeEmpty;
                t.rcnt[s] = 0u;
            }
        }
        SweepWin w0{};
        if (!DIST) {
            hbase = __shfl_sync(0xffffffffu, hbase, 0);
            w0.f = (uint32_t)((hbase + lane) % b.n_frames);
            w0.q = __ldcg(b.frame_page + w0.f);
        }
        const bool valid = p >= 0 && (uint32_t)p < b.n_logical;
        const uint32_t peers = __match_any_sync(0xffffffffu, valid ? (uint32_t)p : 0x80000000u + lane);
        const uint32_t leader = (uint32_t)__ffs((int)peers) - 1u;
        const int32_t rv = ri >= 0 ? __ldcg(release_of + ri) : -1;
        const uint32_t rpeers = __match_any_sync(0xffffffffu, rv >= 0 ? (uint32_t)rv : 0x80000000u + lane);
        // releases by page name pages outside the table's range as bad here
        const bool rin = rv >= 0 && (!BYPAGE || (uint32_t)rv < b.n_logical);
        if (BYPAGE && rv >= 0 && !rin && (uint32_t)(__ffs((int)rpeers) - 1) == lane) bad += (uint32_t)__popc(rpeers);
        __syncthreads();   // tables clear
        uint32_t fslot = kMergeEmpty, rslot = kMergeEmpty;
        if (valid && lane == leader) fslot = merge_insert(t.fkey, t.fcnt, (uint32_t)p, (uint32_t)__popc(peers));
        if (rin && (uint32_t)(__ffs((int)rpeers) - 1) == lane)
            rslot = BYPAGE ? merge_insert(t.fkey, t.frel, (uint32_t)rv, (uint32_t)__popc(rpeers))
                           : merge_insert(t.rkey, t.rcnt, (uint32_t)rv, (uint32_t)__popc(rpeers));
        __syncthreads();   // counts complete
        if (!DIST) w0.e = w0.q < b.n_logical ? __ldcg(b.pt + w0.q) : 0ull;
        // the page's fetch leader moves the block's pins of it with one atomic
        const bool lead = fslot != kMergeEmpty && (fslot & kMergeFirst);
        const uint32_t fs = fslot & ~kMergeFirst;
        const uint32_t k = lead ? t.fcnt[fs] : 0u;
        const uint32_t kr = (BYPAGE && lead) ? t.frel[fs] : 0u;
        unsigned long long fold = 0;
        if (lead) fold = atomicAdd(b.pt + p, (unsigned long long)k - (unsigned long long)kr);
        // releases the fetches did not take along
        const uint32_t rs = rslot & ~kMergeFirst;
        uint32_t rq = 0, rk = 0;
        int32_t rf = -1;
        bool rlead = rslot != kMergeEmpty && (rslot & kMergeFirst);
        if (BYPAGE && rlead && t.fcnt[rs] != 0u) rlead = false;
        if (rlead) {
            rk = BYPAGE ? t.frel[rs] : t.rcnt[rs];
            rlead = release_target<BYPAGE>(b, rv, rk, &rq, &rf, bad);
        }
        unsigned long long rold = 0;
        if (rlead) rold = release_issue(b, rq, rk);
        const uint32_t slot = (slot0 + (uint32_t)i) % b.n_arms;
        int32_t f = -1;
        int st = 0;
        if (lead) {
            if (kr) {
                if (e_frame(fold) < 0 || e_pins(fold) < kr) {   // the releases held no such pins
                    atomicAdd(b.pt + p, (unsigned long long)kr);
                    bad += kr;
                } else {
                    ok += kr;
                    fold -= kr;   // the entry after the releases, before the fetches' pins
                }
            }
            st = fetch_state(b, (uint32_t)p, fold, &f);
        }
        if (rlead) release_check(b, rq, rf, rk, rold, ok, bad);
        if (st == kStHit) acc.hits += k;
        if constexpr (!DIST) {
            // the single hand's loaders of the warp sweep together, starting
            // with the window taken above
            w0.cand = judge(b, w0.f, w0.q, w0.e);
            const uint32_t lm = __ballot_sync(0xffffffffu, st == kStLoad);
            uint32_t old_page = kEmptyPage;
            const int32_t h = sweep_warp(b, lm, (uint32_t)p, &old_page, &w0);
            if (lm) finish_loads_warp<COPY>(b, st == kStLoad, (uint32_t)p, h, old_page, k, acc);
            if (st == kStLoad) f = h;
        } else if (st == kStLoad) {
            uint32_t old_page = kEmptyPage;
            const int32_t h = sweep_private(b, (uint32_t)p, slot, &old_page);
            if (COPY && h >= 0) copy_frame(b, (uint32_t)p, h);
            publish(b, (uint32_t)p, h, old_page, k, acc);
            f = h;
        }
        if (st == kStWait) {
            f = wait_loaded(b, (uint32_t)p);
            if (f >= 0) {
                acc.hits += k;
            } else {
                leave(b, (uint32_t)p, k);
                if (f == kLoading) {
                    acc.timeouts += k;
                    f = -1;
                } else {
                    f = fetch_k<DIST>(b, (uint32_t)p, slot, k, acc);   // the load failed: try once more
                }
            }
        }
        if (lead) t.fres[fs] = f;
        __syncthreads();   // results in the table
        const uint32_t my_slot = __shfl_sync(0xffffffffu, fslot, (int)leader) & ~kMergeFirst;
        if (i < n) {
            const int32_t got = valid ? t.fres[my_slot] : -1;
            frames_out[i] = got;
            if (held_out) held_out[i] = got >= 0 ? p : -1;
        }
        __syncthreads();   // the tables are reused by the next iteration
    }
}

// A round of releases only (no fetch): the lanes of a warp that release
// one name merge into one atomic, and no sweep runs, so the hand stays where
// it is.  BYPAGE as for k_round.
template <bool BYPAGE>
__global__ void __launch_bounds__(256, 4) k_release(BmView b, const int32_t* release_of, const int32_t* release_idx,
                                                 uint32_t n_release) {
    unsigned long long ok = 0, bad = 0;
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    // warp-uniform trip count (blockDim is a multiple of 32)
    for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x - lane; base < n_release; base += stride) {
        const uint64_t j = base + lane;
        const int32_t rv = j < n_release ? __ldcg(release_of + __ldg(release_idx + j)) : -1;
        const uint32_t peers = __match_any_sync(0xffffffffu, rv >= 0 ? (uint32_t)rv : 0x80000000u + lane);
        uint32_t q = 0;
        int32_t f = -1;
        const uint32_t k = (uint32_t)__popc(peers);
        if (rv >= 0 && (uint32_t)(__ffs((int)peers) - 1) == lane && release_target<BYPAGE>(b, rv, k, &q, &f, bad))
            release_check(b, q, f, k, release_issue(b, q, k), ok, bad);
    }
    block_add_counters<2>({ok, bad}, {&b.stats->unpins, &b.stats->bad_unpins});
}

// One round: release the listed pins, then fetch this round's pages.
// With one thread this is the deterministic replay of the round.
// DIST: per-slot hands (b.dist), else the single shared hand.  BYPAGE:
// release_of names pages, else frames.  COPY: misses copy their page from
// the backing store (b.backing and b.frames set).  held_out (may be null)
// receives each fetch's page, or -1 where the fetch got no frame.
template <bool DIST, bool BYPAGE, bool COPY>
__global__ void __launch_bounds__(256) k_round(BmView b, const int32_t* release_of, const int32_t* release_idx,
                                               uint32_t n_release, const int32_t* pages, uint32_t n, uint32_t slot0,
                                               int32_t* frames_out, int32_t* held_out) {
    unsigned long long ok = 0, bad = 0;
    BmAcc acc;
    if ((uint64_t)gridDim.x * blockDim.x == 1u) {
        for (uint32_t j = 0; j < n_release; ++j) {
            uint32_t q;
            int32_t fr;
            if (release_target<BYPAGE>(b, release_of[release_idx[j]], 1u, &q, &fr, bad))
                release_check(b, q, fr, 1u, release_issue(b, q, 1u), ok, bad);
        }
        __threadfence();
        for (uint32_t i = 0; i < n; ++i) {
            int32_t p = pages[i];
            int32_t f = -1;
            if (p >= 0 && (uint32_t)p < b.n_logical) f = fetch_k<DIST>(b, (uint32_t)p, (slot0 + i) % b.n_arms, 1u, acc);
            frames_out[i] = f;
            if (held_out) held_out[i] = f >= 0 ? p : -1;
        }
    } else {
        round_blocks<DIST, BYPAGE, COPY>(b, release_of, release_idx, n_release, pages, n, slot0, frames_out, held_out, ok,
                                   bad, acc);
    }
    block_add_counters<7>({ok, bad, acc.hits, acc.misses, acc.evictions, acc.failures, acc.timeouts},
                          {&b.stats->unpins, &b.stats->bad_unpins, &b.stats->hits, &b.stats->misses,
                           &b.stats->evictions, &b.stats->failures, &b.stats->timeouts});
}

__global__ void k_bm_init(BmView b) {
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t nthr = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t p = tid; p < b.n_logical; p += nthr) b.pt[p] = kEntryNotResident;
    for (uint64_t f = tid; f < b.n_frames; f += nthr) b.frame_page[f] = kEmptyPage;
    for (uint64_t a = tid; a < b.n_arms; a += nthr)
        b.arms[a] = (uint32_t)(((unsigned long long)a * b.n_frames) / b.n_arms);
    if (tid == 0) *b.single_hand = 0ull;
}

// Consistency check: the entries and frame_page are inverse maps, nothing is
// left loading, pins sum.
struct BmCheck {
    unsigned long long resident, mapped_frames, mismatches, loading, pins;
};

__global__ void k_bm_check(BmView b, BmCheck* out) {
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t nthr = (uint64_t)gridDim.x * blockDim.x;
    unsigned long long res = 0, mapped = 0, mism = 0, loading = 0, pins = 0;
    for (uint64_t p = tid; p < b.n_logical; p += nthr) {
        const unsigned long long e = b.pt[p];
        const int32_t f = e_frame(e);
        pins += e_pins(e);
        if (f == kLoading || f == kFailed) { ++loading; continue; }
        if (f < 0) {
            if (e_pins(e) || e_ref(e)) ++mism;   // pins or a reference bit on a page no frame holds
            continue;
        }
        ++res;
        if ((uint32_t)f >= b.n_frames || b.frame_page[f] != p) ++mism;
    }
    for (uint64_t f = tid; f < b.n_frames; f += nthr) {
        const uint32_t pg = b.frame_page[f];
        if (pg == kEmptyPage) continue;
        ++mapped;
        if (pg >= b.n_logical || e_frame(b.pt[pg]) != (int32_t)f) ++mism;
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
    int device;   // the device current at create: every later call runs there
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
    cudaGetDevice(&m->device);
    BmView& b = m->v;
    b.n_logical = (uint32_t)cfg->n_logical;
    b.n_frames = cfg->n_frames;
    b.frame_size = cfg->frame_size;
    b.max_sweep = cfg->max_sweep ? cfg->max_sweep : 2u * cfg->n_frames + 64u;
    b.n_arms = cfg->n_arms ? cfg->n_arms : 1u;
    b.dist = cfg->policy;
    b.backing = (const char*)d_backing;
    bool ok = cudaMalloc(&b.pt, sizeof(unsigned long long) * b.n_logical) == cudaSuccess &&
              cudaMalloc(&b.frame_page, sizeof(uint32_t) * b.n_frames) == cudaSuccess &&
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
    pbm::DeviceScope scope(m->device);
    cudaDeviceSynchronize();
    cudaFree(m->v.pt);
    cudaFree(m->v.frame_page);
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
    pbm::DeviceScope scope(m->device);
    cudaStream_t s = (cudaStream_t)stream;
    k_bm_init<<<sm_count() * 4, 256, 0, s>>>(m->v);
    PBM_LAUNCH_CHECK();
    PBM_CUDA_TRY(cudaMemsetAsync(m->v.stats, 0, sizeof(BmStats), s));
    return PBM_OK;
}

}  // extern "C"

namespace {

int launch_round(pbm_bufmgr* m, bool by_page, const int32_t* d_release_of, const int32_t* d_release_idx,
                 uint32_t n_release, const int32_t* d_pages, uint32_t n, uint32_t slot0, int32_t* d_frames_out,
                 int32_t* d_held_out, int serial, void* stream) {
    if (!m || (n_release && (!d_release_of || !d_release_idx)) || (n && (!d_pages || !d_frames_out)))
        return PBM_ERR_INVALID;
    pbm::DeviceScope scope(m->device);
    if (n == 0 && n_release == 0) return PBM_OK;
    const uint32_t work = n > n_release ? n : n_release;
    const int block = serial ? 1 : 256;
    const int grid = serial ? 1 : (int)((work + 255u) / 256u);
    cudaStream_t s = (cudaStream_t)stream;
    if (n == 0 && !serial) {   // releases only: no fetch, no sweep
        const int rgrid = (int)((n_release + 255u) / 256u);
        if (by_page)
            k_release<true><<<rgrid, 256, 0, s>>>(m->v, d_release_of, d_release_idx, n_release);
        else
            k_release<false><<<rgrid, 256, 0, s>>>(m->v, d_release_of, d_release_idx, n_release);
        PBM_LAUNCH_CHECK();
        return PBM_OK;
    }
    auto go = [&](auto kernel) {
        kernel<<<grid, block, 0, s>>>(m->v, d_release_of, d_release_idx, n_release, d_pages, n, slot0, d_frames_out,
                                      d_held_out);
    };
    const bool copy = m->v.backing && m->v.frames;
    if (copy) {
        if (m->v.dist)
            by_page ? go(k_round<true, true, true>) : go(k_round<true, false, true>);
        else
            by_page ? go(k_round<false, true, true>) : go(k_round<false, false, true>);
    } else {
        if (m->v.dist)
            by_page ? go(k_round<true, true, false>) : go(k_round<true, false, false>);
        else
            by_page ? go(k_round<false, true, false>) : go(k_round<false, false, false>);
    }
    PBM_LAUNCH_CHECK();
    return PBM_OK;
}

}  // namespace

extern "C" {

int pbm_bufmgr_round(pbm_bufmgr* m, const int32_t* d_frames_of, const int32_t* d_release_idx,
                     uint32_t n_release, const int32_t* d_pages, uint32_t n, uint32_t slot0,
                     int32_t* d_frames_out, int serial, void* stream) {
    return launch_round(m, false, d_frames_of, d_release_idx, n_release, d_pages, n, slot0, d_frames_out, nullptr,
                        serial, stream);
}

int pbm_bufmgr_round_pages(pbm_bufmgr* m, const int32_t* d_pages_of, const int32_t* d_release_idx,
                           uint32_t n_release, const int32_t* d_pages, uint32_t n, uint32_t slot0,
                           int32_t* d_frames_out, int32_t* d_held_out, int serial, void* stream) {
    return launch_round(m, true, d_pages_of, d_release_idx, n_release, d_pages, n, slot0, d_frames_out, d_held_out,
                        serial, stream);
}

int pbm_bufmgr_stats(pbm_bufmgr* m, pbm_bufmgr_counters* h_out, void* stream) {
    if (!m || !h_out) return PBM_ERR_INVALID;
    pbm::DeviceScope scope(m->device);
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
    pbm::DeviceScope scope(m->device);
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
    pbm::DeviceScope scope(m->device);
    if (n == 0) return PBM_OK;
    k_bm_gather<<<sm_count() * 4, 256, 0, (cudaStream_t)stream>>>(m->v, d_frame_ids, n, bytes_per_frame / 4u,
                                                                  d_out);
    PBM_LAUNCH_CHECK();
    return PBM_OK;
}

int pbm_bufmgr_read_tables(pbm_bufmgr* m, uint64_t* h_page_entries, uint32_t* h_frame_pages, void* stream) {
    if (!m || (!h_page_entries && !h_frame_pages)) return PBM_ERR_INVALID;
    pbm::DeviceScope scope(m->device);
    cudaStream_t s = (cudaStream_t)stream;
    if (h_page_entries)
        PBM_CUDA_TRY(cudaMemcpyAsync(h_page_entries, m->v.pt, sizeof(uint64_t) * m->v.n_logical,
                                     cudaMemcpyDeviceToHost, s));
    if (h_frame_pages)
        PBM_CUDA_TRY(cudaMemcpyAsync(h_frame_pages, m->v.frame_page, sizeof(uint32_t) * m->v.n_frames,
                                     cudaMemcpyDeviceToHost, s));
    PBM_CUDA_TRY(cudaStreamSynchronize(s));
    return PBM_OK;
}

int pbm_bufmgr_frames(pbm_bufmgr* m, void** d_frames, size_t* bytes) {
    if (!m) return PBM_ERR_INVALID;
    if (d_frames) *d_frames = m->v.frames;
    if (bytes) *bytes = m->frames_bytes;
    return PBM_OK;
}

}  // extern "C"
