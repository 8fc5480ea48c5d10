// Harness for source/CRW_BM.cuh (clustered walk).
#include "fx_common.cuh"
#include "CRW_BM.cuh"

extern "C" __global__ void fx_setup(int* words, int n_words, int n_pages, int* last_group,
                                    int8_t* last_bit) {
    d_PageMapRandomWalk_BM = words;
    Bitmap_length_d = n_words;
    d_total_n_pages = n_pages;
    d_LastFreeGroup = last_group;
    d_LastFreeBit = last_bit;
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
