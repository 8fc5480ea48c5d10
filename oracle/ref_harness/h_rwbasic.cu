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

extern "C" __global__ void fx_free_seq(int n, const int* ids) {
    if (fx_tid() != 0) return;
    for (int k = 0; k < n; ++k) freePage(ids[k]);
}
