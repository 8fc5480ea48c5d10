// First translation unit of a two-unit caller of the -rdc drop-in: it takes
// pages with the collaborative bitmap walk and writes each owner's index
// into its page.  The second unit (pp_rdc_free.cu) frees them.
#define PBM_PARALLELPAGE_RDC
#include "pbm/parallelPage.cuh"

__global__ void rdc_get_kernel(int n, int* ids) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int id = getPageCollabRW_BM();
    ids[t] = id;
    if (id >= 0) ((int*)pageAddress(id))[0] = t;
}

extern "C" void rdc_alloc(int n, int* d_ids) {
    rdc_get_kernel<<<(n + 127) / 128, 128>>>(n, d_ids);
    cudaDeviceSynchronize();
}
