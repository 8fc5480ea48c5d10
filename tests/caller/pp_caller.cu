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

// the strategy (index in parallelPage.cuh's order) each case draws from
static int pool_of(int which) {
    static const int map[12] = {0, 1, 2, 3, 4, 5, 6, 7, 8, 7, 6, 8};
    return map[which];
}

// out: [0] bad, [1] free pages before, [2] after get, [3] after free
extern "C" int pp_run(int which, int n, int* h_ids, long long* out) {
    typedef void (*init_t)();
    static const init_t inits[9] = {initPagesRandomWalk, initPagesClusteredRandomWalk, initPagesLinkedList,
                                    initPagesSingleClock, initPagesDistClock, initPagesCollabRW,
                                    initPagesCollabRW_BM, initPagesRandomWalk_BM,
                                    initPagesClusteredRandomWalk_BM};
    const int k = pool_of(which);
    if (pbmFreePagesLeft(k) == 0) inits[k]();
    int *d_ids, *d_steps, *d_bad;
    cudaMalloc(&d_ids, n * 4);
    cudaMalloc(&d_steps, n * 4);
    cudaMalloc(&d_bad, 4);
    cudaMemset(d_bad, 0, 4);
    out[1] = (long long)pbmFreePagesLeft(k);
    get_kernel<<<(n + 127) / 128, 128>>>(n, which, d_ids, d_steps);
    cudaDeviceSynchronize();
    out[2] = (long long)pbmFreePagesLeft(k);
    check_free_kernel<<<(n + 127) / 128, 128>>>(n, which, d_ids, d_bad);
    cudaDeviceSynchronize();
    out[3] = (long long)pbmFreePagesLeft(k);
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

// The nine strategies share one page store: a payload written through
// pageAddress for a page of the first strategy reads back the same after
// the other eight are initialised, and initialising them takes far less
// device memory than another store.  out: [0] bytes the eight took,
// [1] payload read back, [2] the store's bytes
__global__ void pp_store_get(int* id_out) {
    const int id = getPageRandomWalk();
    *id_out = id;
    if (id >= 0) ((int*)pageAddress(id))[0] = 0x5A5A1234;
}
__global__ void pp_store_read(const int* id_in, int* v_out) {
    const int id = *id_in;
    *v_out = id >= 0 ? ((const int*)pageAddress(id))[0] : -1;
}
extern "C" int pp_shared_store(long long* out) {
    initPagesRandomWalk();
    int* d = nullptr;
    if (cudaMalloc(&d, 2 * sizeof(int)) != cudaSuccess) return -1;
    pp_store_get<<<1, 1>>>(d);
    cudaDeviceSynchronize();
    size_t free0 = 0, free1 = 0, total = 0;
    cudaMemGetInfo(&free0, &total);
    initPagesClusteredRandomWalk();
    initPagesLinkedList();
    initPagesSingleClock();
    initPagesDistClock();
    initPagesCollabRW();
    initPagesCollabRW_BM();
    initPagesRandomWalk_BM();
    initPagesClusteredRandomWalk_BM();
    cudaDeviceSynchronize();
    cudaMemGetInfo(&free1, &total);
    pp_store_read<<<1, 1>>>(d, d + 1);
    int v = 0;
    cudaMemcpy(&v, d + 1, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(d);
    out[0] = (long long)free0 - (long long)free1;
    out[1] = v;
    out[2] = (long long)TOTAL_N_PAGES * PAGE_SIZE;
    return cudaGetLastError() == cudaSuccess ? 0 : -2;
}
