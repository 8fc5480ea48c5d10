// Harness for source/RandomWalkBasic.cuh (getPage/freePage on an int map).
#include "fx_common.cuh"
#include "RandomWalkBasic.cuh"

extern "C" __global__ void fx_setup(int* map, int n_pages) {
    d_PageMapRandomWalkBasic = map;
    d_total_n_pages = n_pages;
}

// Thread `tid` calls getPage n times, clock fixed to clocks[k] for call k.
extern "C" __global__ void fx_get_seq(int tid, int n, const int* clocks, int* ids, int* steps) {
    if (fx_tid() != tid) return;
    for (int k = 0; k < n; ++k) {
        fx_clock_val = clocks[k];
        int s = 0;
        ids[k] = getPage(&s);
        steps[k] = s;
    }
}

// Churn for timing: thread i releases the page in arena slot (off + i) mod H,
// then takes a new one with getPage (see h_collab.cu).
extern "C" __global__ void fx_churn(int n, int* arena, int H, int off) {
    const int i = fx_tid();
    if (i >= n) return;
    int slot = off + i;
    if (slot >= H) slot -= H;
    freePage(arena[slot]);
    int s = 0;
    arena[slot] = getPage(&s);
}

extern "C" __global__ void fx_free_seq(int n, const int* ids) {
    if (fx_tid() != 0) return;
    for (int k = 0; k < n; ++k) freePage(ids[k]);
}
