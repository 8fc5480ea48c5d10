// A caller of the reference's MemoryManager classes (unitTests/unitTestMalloc1.cu
// shape: random sizes from a per-thread LCG), compiled against pbm/malloc.cuh.
#define PBM_MALLOC_POOL_PAGES (1u << 18)
#include <type_traits>

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

// KernelMallocSimple: each thread lets go of its chunk once its blocks are freed
template <class MM>
__global__ void retire_kernel(MM mm, int n) {
    int tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= n) return;
    if constexpr (std::is_same<MM, KernelMallocSimple>::value) mm.retire();
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
    retire_kernel<<<(n + 127) / 128, 128>>>(mm, n);
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

// KernelMallocSimple's bump order: three 40-byte mallocs of one thread are
// consecutive 48-byte slices of its chunk; different threads' chunks never
// overlap; after the frees and retire() every page is back.
// out: [0] bad, [1] free fraction before (x1e6), [2] after the mallocs, [3] after free + retire
__global__ void bump_kernel(KernelMallocSimple mm, int n, unsigned long long* ptrs) {
    int tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= n) return;
    for (int k = 0; k < 3; ++k) {
        int* p = (int*)mm.malloc(40);
        ptrs[tid * 3 + k] = (unsigned long long)p;
        if (p) for (int j = 0; j < 10; ++j) p[j] = tid * 3 + k;
    }
}
__global__ void bump_check_kernel(KernelMallocSimple mm, int n, const unsigned long long* ptrs, int* bad) {
    int tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= n) return;
    const unsigned long long p0 = ptrs[tid * 3];
    for (int k = 0; k < 3; ++k) {
        const int* p = (const int*)ptrs[tid * 3 + k];
        if (!p || ptrs[tid * 3 + k] != p0 + 48ull * k) { atomicAdd(bad, 1); continue; }
        for (int j = 0; j < 10; ++j)
            if (p[j] != tid * 3 + k) { atomicAdd(bad, 1); break; }
        mm.free((void*)p);
    }
    mm.retire();
}
extern "C" int malloc_bump_run(int n, long long* out) {
    KernelMallocSimple mm(n);
    unsigned long long* d_ptrs;
    int* d_bad;
    cudaMalloc(&d_ptrs, 3ull * n * 8);
    cudaMalloc(&d_bad, 4);
    cudaMemset(d_bad, 0, 4);
    float f0 = mm.freePagePercentage();
    bump_kernel<<<(n + 127) / 128, 128>>>(mm, n, d_ptrs);
    cudaDeviceSynchronize();
    float f1 = mm.freePagePercentage();
    bump_check_kernel<<<(n + 127) / 128, 128>>>(mm, n, d_ptrs, d_bad);
    cudaDeviceSynchronize();
    float f2 = mm.freePagePercentage();
    int bad = 0;
    cudaMemcpy(&bad, d_bad, 4, cudaMemcpyDeviceToHost);
    out[0] = bad;
    out[1] = (long long)(f0 * 1e6 + 0.5);
    out[2] = (long long)(f1 * 1e6 + 0.5);
    out[3] = (long long)(f2 * 1e6 + 0.5);
    cudaFree(d_ptrs);
    cudaFree(d_bad);
    mm.release();
    return cudaGetLastError() == cudaSuccess ? 0 : -2;
}
