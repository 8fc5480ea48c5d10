// A caller's translation unit written against the reference's header-only API
// (the shape of unitTests/unitTest1.cu and unitTest1.5.cu), compiled against
// the drop-in header named by PBM_FAMILY_HEADER and linked with -lpbm.
#include PBM_FAMILY_HEADER

__global__ void get1page_kernel(int Nthreads, int* d_step_counts, int* d_ids) {
    int tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid < Nthreads) {
        int step_counts = 0;
        int pageID = getPage(&step_counts);
        d_ids[tid] = pageID;
        if (d_step_counts) d_step_counts[tid] = step_counts;
        if (pageID >= 0) ((int*)pageAddress(pageID))[0] = tid;
    }
}

__global__ void check_kernel(int Nthreads, const int* d_ids, int* d_bad) {
    int tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid < Nthreads) {
        int id = d_ids[tid];
        if (id < 0) { atomicAdd(d_bad, 1); return; }
        void* p = pageAddress(id);
        if (((int*)p)[0] != tid) atomicAdd(d_bad, 1);
        if (getPageID(p) != id) atomicAdd(d_bad, 1);
    }
}

__global__ void freePage_kernel(int Nthreads, const int* d_ids) {
    int tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid < Nthreads) freePage(d_ids[tid]);
}

// out: [0] failed ids + bad payloads, [1..4] free fraction before alloc,
// after alloc, after free, after reset (x 1e6, rounded), [5] pages, [6] sum of steps
extern "C" int dropin_run(int nGB, int pageSize, float prefillFree, int n, int block, long long* out) {
    initMemoryManagement(nGB, pageSize);
    prefillBuffer(prefillFree);
    int *d_ids = nullptr, *d_steps = nullptr, *d_bad = nullptr;
    cudaMalloc(&d_ids, n * sizeof(int));
    cudaMalloc(&d_steps, n * sizeof(int));
    cudaMalloc(&d_bad, sizeof(int));
    cudaMemset(d_bad, 0, sizeof(int));
    float f0 = getFreePagePercentage();
    get1page_kernel<<<(n + block - 1) / block, block>>>(n, d_steps, d_ids);
    check_kernel<<<(n + 255) / 256, 256>>>(n, d_ids, d_bad);
    cudaDeviceSynchronize();
    float f1 = getFreePagePercentage();
    freePage_kernel<<<(n + block - 1) / block, block>>>(n, d_ids);
    cudaDeviceSynchronize();
    float f2 = getFreePagePercentage();
    int bad = 0;
    cudaMemcpy(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost);
    int* h_steps = new int[n];
    cudaMemcpy(h_steps, d_steps, n * sizeof(int), cudaMemcpyDeviceToHost);
    long long ssum = 0;
    for (int i = 0; i < n; ++i) ssum += h_steps[i];
    delete[] h_steps;
    resetMemoryManager();
    float f3 = getFreePagePercentage();
    out[0] = bad;
    out[1] = (long long)(f0 * 1e6 + 0.5);
    out[2] = (long long)(f1 * 1e6 + 0.5);
    out[3] = (long long)(f2 * 1e6 + 0.5);
    out[4] = (long long)(f3 * 1e6 + 0.5);
    out[5] = h_total_n_pages;
    out[6] = ssum;
    cudaFree(d_ids);
    cudaFree(d_steps);
    cudaFree(d_bad);
    return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

#ifdef PBM_WITH_MALLOC
// mallocRW / freeRW from a caller's kernels (unitTests/unitTest3.cu shape):
// every thread takes a block, fills it with its id, and frees it later.
__global__ void malloc_kernel(int n, const int* sizes, unsigned long long* ptrs) {
    int tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid < n) {
        void* p = mallocRW((size_t)sizes[tid]);
        ptrs[tid] = (unsigned long long)p;
        if (p) {
            int* q = (int*)p;
            for (int k = 0; k < sizes[tid] / 4; ++k) q[k] = tid;
        }
    }
}

__global__ void malloc_check(int n, const int* sizes, const unsigned long long* ptrs, int* bad) {
    int tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid < n) {
        const int* q = (const int*)ptrs[tid];
        if (!q) { atomicAdd(bad, 1); return; }
        for (int k = 0; k < sizes[tid] / 4; ++k)
            if (q[k] != tid) { atomicAdd(bad, 1); return; }
    }
}

__global__ void mfree_kernel(int n, const unsigned long long* ptrs) {
    int tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid < n) freeRW((void*)ptrs[tid]);
}

// out: [0] failed or overwritten blocks, [1] free fraction before (x1e6),
// [2] after malloc, [3] after free
extern "C" int dropin_malloc_run(int nGB, int pageSize, int n, const int* h_sizes, long long* out) {
    initMemoryManagement(nGB, pageSize);
    int *d_sizes = nullptr, *d_bad = nullptr;
    unsigned long long* d_ptrs = nullptr;
    cudaMalloc(&d_sizes, n * sizeof(int));
    cudaMalloc(&d_ptrs, n * sizeof(unsigned long long));
    cudaMalloc(&d_bad, sizeof(int));
    cudaMemcpy(d_sizes, h_sizes, n * sizeof(int), cudaMemcpyHostToDevice);
    cudaMemset(d_bad, 0, sizeof(int));
    float f0 = getFreePagePercentage();
    malloc_kernel<<<(n + 63) / 64, 64>>>(n, d_sizes, d_ptrs);
    malloc_check<<<(n + 255) / 256, 256>>>(n, d_sizes, d_ptrs, d_bad);
    cudaDeviceSynchronize();
    float f1 = getFreePagePercentage();
    mfree_kernel<<<(n + 63) / 64, 64>>>(n, d_ptrs);
    cudaDeviceSynchronize();
    float f2 = getFreePagePercentage();
    int bad = 0;
    cudaMemcpy(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost);
    out[0] = bad;
    out[1] = (long long)(f0 * 1e6 + 0.5);
    out[2] = (long long)(f1 * 1e6 + 0.5);
    out[3] = (long long)(f2 * 1e6 + 0.5);
    cudaFree(d_sizes);
    cudaFree(d_ptrs);
    cudaFree(d_bad);
    return cudaGetLastError() == cudaSuccess ? 0 : -2;
}
#endif
