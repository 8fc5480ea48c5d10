// Harness for source/CollabRW_BM.cuh (warp-collaborative walk).
#include "fx_common.cuh"
#include "CollabRW_BM.cuh"

extern "C" __global__ void fx_setup(int* words, int n_words, int n_pages) {
    d_PageMapRandomWalk_BM = words;
    Bitmap_length_d = n_words;
    d_total_n_pages = n_pages;
}

// Churn for timing: thread i releases the page held in arena slot
// (off + i) mod H with the reference's freePage, then takes a new one with its
// getPage and stores it in the slot.  Releasing first keeps the free pages at
// or above their starting count, so the walk (which spins until it finds a
// page) always has pages to find while the caller keeps n well below them.
extern "C" __global__ void fx_churn(int n, int* arena, int H, int off) {
    const int i = fx_tid();
    if (i >= n) return;
    int slot = off + i;
    if (slot >= H) slot -= H;
    freePage(arena[slot]);
    int s = 0;
    arena[slot] = getPage(&s);
}

// One warp (launch <<<1,32>>>); for call k the lanes in masks[k] call getPage.
extern "C" __global__ void fx_collab_seq(int n, const int* clocks, const unsigned* masks, int* ids,
                                         int* steps) {
    const int lane = threadIdx.x & 31;
    for (int k = 0; k < n; ++k) {
        if (lane == 0) fx_clock_val = clocks[k];
        __syncwarp();
        __threadfence_block();
        if (masks[k] & (1u << lane)) {
            int s = 0;
            int id = getPage(&s);
            ids[k * 32 + lane] = id;
            steps[k * 32 + lane] = s;
        }
        __syncwarp();
    }
}
