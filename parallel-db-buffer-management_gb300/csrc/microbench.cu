// microbench.cu -- uncontended atomicOr ceiling (the roofline denominator of
// the allocation kernels, whose bitmaps live in L2).
//
// Every thread issues `iters` atomicOr operations, each to a word no other
// thread touches in the same iteration.  Two address patterns are timed and
// the faster one is the ceiling:
//   line:    the 32 lanes of a warp hit the 32 words of one 128-byte line
//            (what a collaborative walk does);
//   spread:  neighbouring lanes are 33 words apart, so one warp instruction
//            touches 32 different lines and L2 slices (what frees of random
//            pages do).
// The reference's precedent is its atomicExch lock microbenchmark
// (unitTests/unitTestLinkedList2.cu:3-16).
#include "internal.cuh"

namespace pbm {

template <bool kReturning, bool kSpread>
__global__ void __launch_bounds__(256) k_atomic_ceiling(uint32_t* buf, uint32_t mask, uint32_t iters,
                                                        uint32_t* sink) {
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nthr = gridDim.x * blockDim.x;
    uint32_t acc = 0;
    for (uint32_t i = 0; i < iters; ++i) {
        uint32_t slot = tid + i * nthr;
        uint32_t w = kSpread ? ((slot >> 5) * 32u * 33u + (slot & 31u) * 33u) & mask : slot & mask;
        uint32_t bit = 1u << (i & 31u);
        if (kReturning) acc ^= atomicOr(buf + w, bit);
        else atomicOr(buf + w, bit);
    }
    if (kReturning && acc == 0x9E3779B9u) sink[0] = acc;
}

template <bool R, bool S>
static int time_one(uint32_t* buf, uint32_t mask, uint32_t threads, uint32_t iters, uint32_t* sink,
                    float* ms) {
    const int block = 256;
    const uint32_t grid = (threads + block - 1) / block;
    cudaEvent_t e0, e1;
    PBM_CUDA_TRY(cudaEventCreate(&e0));
    PBM_CUDA_TRY(cudaEventCreate(&e1));
    k_atomic_ceiling<R, S><<<grid, block>>>(buf, mask, iters, sink);  // warm-up
    PBM_LAUNCH_CHECK();
    float best = 1e30f;
    for (int rep = 0; rep < 5; ++rep) {
        PBM_CUDA_TRY(cudaEventRecord(e0, 0));
        k_atomic_ceiling<R, S><<<grid, block>>>(buf, mask, iters, sink);
        PBM_LAUNCH_CHECK();
        PBM_CUDA_TRY(cudaEventRecord(e1, 0));
        PBM_CUDA_TRY(cudaEventSynchronize(e1));
        float t = 0;
        PBM_CUDA_TRY(cudaEventElapsedTime(&t, e0, e1));
        if (t < best) best = t;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms = best;
    return PBM_OK;
}

}  // namespace pbm

using namespace pbm;

extern "C" int pbm_atomic_ceiling(uint32_t words, uint32_t threads, uint32_t iters, int returning,
                                  int pattern, double* h_ops_per_s, double* h_ms) {
    if (!h_ops_per_s || words < 1024 || (words & (words - 1)) || threads == 0 || iters == 0 ||
        pattern < 0 || pattern > 2)
        return PBM_ERR_INVALID;
    uint32_t* buf = nullptr;
    uint32_t* sink = nullptr;
    if (cudaMalloc(&buf, (size_t)words * 4u) != cudaSuccess || cudaMalloc(&sink, 4) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(buf);
        return PBM_ERR_NOMEM;
    }
    PBM_CUDA_TRY(cudaMemset(buf, 0, (size_t)words * 4u));
    float t_line = 1e30f, t_spread = 1e30f;
    int rc = PBM_OK;
    if (pattern != 2)
        rc = returning ? time_one<true, false>(buf, words - 1u, threads, iters, sink, &t_line)
                       : time_one<false, false>(buf, words - 1u, threads, iters, sink, &t_line);
    if (!rc && pattern != 1)
        rc = returning ? time_one<true, true>(buf, words - 1u, threads, iters, sink, &t_spread)
                       : time_one<false, true>(buf, words - 1u, threads, iters, sink, &t_spread);
    cudaFree(buf);
    cudaFree(sink);
    if (rc) return rc;
    const float best = t_line < t_spread ? t_line : t_spread;
    *h_ops_per_s = (double)threads * (double)iters / (best * 1e-3);
    if (h_ms) *h_ms = best;
    return PBM_OK;
}
