// A caller of the reference's monolithic API (parallelPage.cuh), compiled
// against the drop-in pbm/parallelPage.cuh with a smaller compile-time pool.
#define TOTAL_N_PAGES 1000000
#define PAGE_SIZE 256
#include "pbm/parallelPage.cuh"

__global__ void get_kernel(int n, int which, int* ids, int* steps) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    int s = 0, id = -1;
    switch (which) {
    case 0: id = getPageRandomWalk(&s); break;
    case 1: id = getPageClusteredRandomWalk(&s); break;
    case 2: id = getPageLinkedList(&s); break;
    case 3: id = getPageSingleClock(&s); break;
    case 4: id = getPageDistClock(&s); break;
    case 5: id = getPageCollabRW(&s); break;
    case 6: id = getPageCollabRW_BM(&s); break;
    case 7: id = getPageRandomWalk_BM(&s); break;
    case 8: id = getPageClusteredRandomWalk_BM(&s); break;
    case 9: id = getXPageRandomWalk_BM(4, &s); break;
    case 10: id = getXPageCollabRW_BM(3, &s); break;
    case 11: id = getXPageClusteredRandomWalk_BM(2, &s); break;
    }
    ids[t] = id;
    steps[t] = s;
    if (id >= 0) ((int*)pageAddress(id))[0] = t;
}

__global__ void check_free_kernel(int n, int which, const int* ids, int* bad) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    int id = ids[t];
    if (id < 0) { atomicAdd(bad, 1); return; }
    if (((int*)pageAddress(id))[0] != t) atomicAdd(bad, 1);
    switch (which) {
    case 0: freePageRandomWalk(id); break;
    case 1: freePageClusteredRandomWalk(id); break;
    case 2: freePageLinkedList(id); break;
    case 3: freePageSingleClock(id); break;
    case 4: freePageDistClock(id); break;
    case 5: freePageCollabRW(id); break;
    case 6: freePageCollabRW_BM(id); break;
    case 7: freePageRandomWalk_BM(id); break;
    case 8: freePageClusteredRandomWalk_BM(id); break;
    default: break;   // runs are left held
    }
}

static int pool_of(int which) {
    static const int map[12] = {PBM_PP_RW, PBM_PP_CRW, PBM_PP_LL, PBM_PP_SC, PBM_PP_DC, PBM_PP_CORW,
                                PBM_PP_CORW_BM, PBM_PP_RW_BM, PBM_PP_CRW_BM, PBM_PP_RW_BM, PBM_PP_CORW_BM,
                                PBM_PP_CRW_BM};
    return map[which];
}

// out: [0] bad, [1] free pages before, [2] after get, [3] after free
extern "C" int pp_run(int which, int n, int* h_ids, long long* out) {
    typedef void (*init_t)();
    static const init_t inits[PBM_PP_N] = {initPagesRandomWalk, initPagesClusteredRandomWalk, initPagesLinkedList,
                                           initPagesSingleClock, initPagesDistClock, initPagesCollabRW,
                                           initPagesCollabRW_BM, initPagesRandomWalk_BM,
                                           initPagesClusteredRandomWalk_BM};
    const int k = pool_of(which);
    if (!pbm_pp_host[k].pool) inits[k]();
    int *d_ids, *d_steps, *d_bad;
    cudaMalloc(&d_ids, n * 4);
    cudaMalloc(&d_steps, n * 4);
    cudaMalloc(&d_bad, 4);
    cudaMemset(d_bad, 0, 4);
    out[1] = (long long)pbm::dropin::free_pages(pbm_pp_host[k]);
    get_kernel<<<(n + 127) / 128, 128>>>(n, which, d_ids, d_steps);
    cudaDeviceSynchronize();
    out[2] = (long long)pbm::dropin::free_pages(pbm_pp_host[k]);
    check_free_kernel<<<(n + 127) / 128, 128>>>(n, which, d_ids, d_bad);
    cudaDeviceSynchronize();
    out[3] = (long long)pbm::dropin::free_pages(pbm_pp_host[k]);
    int bad = 0;
    cudaMemcpy(&bad, d_bad, 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(h_ids, d_ids, n * 4, cudaMemcpyDeviceToHost);
    out[0] = bad;
    printNumPagesLeftRandomWalk();
    cudaFree(d_ids);
    cudaFree(d_steps);
    cudaFree(d_bad);
    return cudaGetLastError() == cudaSuccess ? 0 : -2;
}
