// A caller of the reference's MemoryManager classes (unitTests/unitTestMalloc1.cu
// shape: random sizes from a per-thread LCG), compiled against pbm/malloc.cuh.
#define PBM_MALLOC_POOL_PAGES (1u << 18)
#include "pbm/malloc.cuh"

template <class MM>
__global__ void malloc_kernel(MM mm, int n, unsigned long long* ptrs, int* sizes) {
    int tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= n) return;
    int size = 4 + (int)(((unsigned)tid * 1103515245u + 12345u) % 8188u);   // 4 .. 8191 bytes
    sizes[tid] = size;
    int* p = (int*)mm.malloc(size);
    ptrs[tid] = (unsigned long long)p;
    if (p) for (int k = 0; k < size / 4; ++k) p[k] = tid;
}

template <class MM>
__global__ void check_free_kernel(MM mm, int n, const unsigned long long* ptrs, const int* sizes, int* bad) {
    int tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= n) return;
    const int* p = (const int*)ptrs[tid];
    if (!p) { atomicAdd(bad, 1); return; }
    for (int k = 0; k < sizes[tid] / 4; ++k)
        if (p[k] != tid) { atomicAdd(bad, 1); break; }
    mm.free((void*)p);
}

template <class MM>
static int run(MM& mm, int n, long long* out) {
    unsigned long long* d_ptrs;
    int *d_sizes, *d_bad;
    cudaMalloc(&d_ptrs, n * 8);
    cudaMalloc(&d_sizes, n * 4);
    cudaMalloc(&d_bad, 4);
    cudaMemset(d_bad, 0, 4);
    float f0 = mm.freePagePercentage();
    malloc_kernel<<<(n + 127) / 128, 128>>>(mm, n, d_ptrs, d_sizes);
    cudaDeviceSynchronize();
    float f1 = mm.freePagePercentage();
    check_free_kernel<<<(n + 127) / 128, 128>>>(mm, n, d_ptrs, d_sizes, d_bad);
    cudaDeviceSynchronize();
    float f2 = mm.freePagePercentage();
    int bad = 0;
    cudaMemcpy(&bad, d_bad, 4, cudaMemcpyDeviceToHost);
    out[0] = bad;
    out[1] = (long long)(f0 * 1e6 + 0.5);
    out[2] = (long long)(f1 * 1e6 + 0.5);
    out[3] = (long long)(f2 * 1e6 + 0.5);
    cudaFree(d_ptrs);
    cudaFree(d_sizes);
    cudaFree(d_bad);
    mm.release();
    return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

extern "C" int malloc_run(int which, int n, long long* out) {
    if (which == 0) {
        KernelMallocSimple mm(n);
        return run(mm, n, out);
    }
    KernelMallocCollab mm;
    return run(mm, n, out);
}
