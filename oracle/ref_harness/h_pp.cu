// Harness for source/parallelPage.cu (monolithic API, TOTAL_N_PAGES fixed at
// compile time by parallelPage.cuh).
#include "fx_common.cuh"
#include "parallelPage.cu"

extern "C" __global__ void fx_setup(int* sc_map, int* dc_map, int* dc_arms, int* rwbm_words,
                                    void* ll_nodes) {
    d_pageMapSingleClock = sc_map;
    d_SingleClockArm = 0;
    d_pageMapDistClock = dc_map;
    d_DistClockArm = dc_arms;
    d_PageMapRandomWalk_BM = rwbm_words;
    d_nodes = (Node_t*)ll_nodes;
}

extern "C" __global__ void fx_total_pages(int* out) { out[0] = TOTAL_N_PAGES; out[1] = BITMAP_LENGTH; }

extern "C" __global__ void fx_single_clock_seq(int n, int* ids, int* steps) {
    if (fx_tid() != 0) return;
    for (int k = 0; k < n; ++k) { int s = 0; ids[k] = getPageSingleClock(&s); steps[k] = s; }
}

// randomizeArmDistClock for thread `tid` with a fixed clock, then n gets.
extern "C" __global__ void fx_dist_clock_seq(int tid, int clk, int n, int* arm0, int* ids, int* steps) {
    if (fx_tid() != tid) return;
    fx_clock_val = clk;
    int16_t Clock = (int16_t)clock();
    int seed = (tid << 15) + Clock;
    seed = RNG_LCG(seed);
    seed = seed % TOTAL_N_PAGES;
    d_DistClockArm[tid] = seed;   // parallelPage.cu:546-555, one thread
    arm0[0] = seed;
    for (int k = 0; k < n; ++k) { int s = 0; ids[k] = getPageDistClock(&s); steps[k] = s; }
}

extern "C" __global__ void fx_getxpage_seq(int tid, int X, int n, const int* clocks, int* ids, int* steps) {
    if (fx_tid() != tid) return;
    for (int k = 0; k < n; ++k) {
        fx_clock_val = clocks[k];
        int s = 0;
        ids[k] = getXPageRandomWalk_BM(X, &s);
        steps[k] = s;
    }
}

// Linked list: ops[k] < 0 -> getPageLinkedList, else freePageLinkedList(ops[k]).
extern "C" __global__ void fx_ll_seq(int n, const int* ops, int* out) {
    if (fx_tid() != 0) return;
    for (int k = 0; k < n; ++k) {
        if (ops[k] < 0) out[k] = getPageLinkedList(nullptr);
        else { freePageLinkedList(ops[k], nullptr); out[k] = -1; }
    }
}

// ---- churn for timing (reference timing arm) ----
// Thread i releases the page held in arena slot (off + i) mod H with the
// strategy's own freePage, then takes a new one with its getPage and stores
// it in the slot.  Releasing first keeps the free pages at or above their
// start, so the unbounded getPage loops always have pages to find while the
// caller keeps each launch well below the free pages.
extern "C" __global__ void fx_churn_sc(int n, int* arena, int H, int off) {
    const int i = fx_tid();
    if (i >= n) return;
    int slot = off + i;
    if (slot >= H) slot -= H;
    freePageSingleClock(arena[slot], nullptr);
    arena[slot] = getPageSingleClock(nullptr);
}

// DistClock indexes its arms by the global thread id, so a launch must stay
// below MAX_THREADS_DISTCLOCK threads (the caller caps it).
extern "C" __global__ void fx_churn_dc(int n, int* arena, int H, int off) {
    const int i = fx_tid();
    if (i >= n) return;
    int slot = off + i;
    if (slot >= H) slot -= H;
    freePageDistClock(arena[slot], nullptr);
    arena[slot] = getPageDistClock(nullptr);
}

// The single clock's arm (an int that must stay far from 2^31) and the
// distributed clock's thread limit.
extern "C" __global__ void fx_sc_arm(int* out) { out[0] = d_SingleClockArm; out[1] = MAX_THREADS_DISTCLOCK; }
