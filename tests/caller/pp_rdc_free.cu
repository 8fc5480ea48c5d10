// Second translation unit of the two-unit -rdc caller: it checks each page's
// payload through pageAddress and frees the pages the first unit took, in
// the same shared map.
#define PBM_PARALLELPAGE_RDC
#include "pbm/parallelPage.cuh"

extern "C" void rdc_alloc(int n, int* d_ids);   // pp_rdc_alloc.cu

__global__ void rdc_free_kernel(int n, const int* ids, int* bad) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int id = ids[t];
    if (id < 0 || ((const int*)pageAddress(id))[0] != t) atomicAdd(bad, 1);
    if (id >= 0) freePageCollabRW_BM(id);
}

// out: [0] bad pages, [1] free before, [2] after the first unit's gets,
// [3] after this unit's frees; ids copied to h_ids
extern "C" int rdc_run(int n, int* h_ids, long long* out) {
    initPagesCollabRW_BM();
    int *d_ids = nullptr, *d_bad = nullptr;
    if (cudaMalloc(&d_ids, n * sizeof(int)) != cudaSuccess || cudaMalloc(&d_bad, sizeof(int)) != cudaSuccess)
        return -1;
    cudaMemset(d_bad, 0, sizeof(int));
    out[1] = (long long)pbmFreePagesLeft(6);
    rdc_alloc(n, d_ids);
    out[2] = (long long)pbmFreePagesLeft(6);
    rdc_free_kernel<<<(n + 127) / 128, 128>>>(n, d_ids, d_bad);
    cudaDeviceSynchronize();
    out[3] = (long long)pbmFreePagesLeft(6);
    int bad = 0;
    cudaMemcpy(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost);
    cudaMemcpy(h_ids, d_ids, n * sizeof(int), cudaMemcpyDeviceToHost);
    out[0] = bad;
    cudaFree(d_ids);
    cudaFree(d_bad);
    return cudaGetLastError() == cudaSuccess ? 0 : -2;
}
