// Harness for source/RandomWalkBasic_BM.cuh (word-probe walk on a 32-bit bitmap).
#include "fx_common.cuh"
#include "RandomWalkBasic_BM.cuh"

extern "C" __global__ void fx_setup(int* words, int n_words, int n_pages) {
    d_PageMapRandomWalk_BM = words;
    Bitmap_length_d = n_words;
    d_total_n_pages = n_pages;
}

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

extern "C" __global__ void fx_lcg(int n, const int* in, int* out) {
    int i = fx_tid();
    if (i < n) out[i] = RNG_LCG(in[i]);
}
