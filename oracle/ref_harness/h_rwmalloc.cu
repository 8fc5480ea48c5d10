// Harness for source/RWMalloc.cuh (find0Range, getNPage).
#include "fx_common.cuh"
#include "RWMalloc.cuh"

extern "C" __global__ void fx_setup(int* words, int n_words, int n_pages) {
    d_PageMapRandomWalk_BM = words;
    Bitmap_length_d = n_words;
    d_total_n_pages = n_pages;
}

extern "C" __global__ void fx_find0range(int n, const int* xs, int* lens, int* starts, int* xs_out) {
    int i = fx_tid();
    if (i >= n) return;
    int x = xs[i], st = -99;
    int len = find0Range(&x, &st);
    lens[i] = len;
    starts[i] = st;
    xs_out[i] = x;
}

// One warp: call k, lanes in masks[k] request npages[k*32+lane] pages.
extern "C" __global__ void fx_getnpage_seq(int n, const int* clocks, const unsigned* masks,
                                           const int* npages, int* ids, int* steps) {
    const int lane = threadIdx.x & 31;
    for (int k = 0; k < n; ++k) {
        if (lane == 0) fx_clock_val = clocks[k];
        __syncwarp();
        __threadfence_block();
        if (masks[k] & (1u << lane)) {
            int s = 0;
            int id = getNPage(npages[k * 32 + lane], &s);
            ids[k * 32 + lane] = id;
            steps[k * 32 + lane] = s;
        }
        __syncwarp();
    }
}
