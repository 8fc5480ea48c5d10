// monitor.cu -- occupancy and statistics sampled while kernels run.
//
// The reference's monitorBufferRandomWalk (parallelPage.cu:209-223) prints
// the number of free pages every msGap milliseconds from a host loop that
// copies the whole map back each time.  Here a host thread samples the pool
// on its own non-blocking stream: a small popcount kernel over the bitmap
// (2 MiB at 2^24 pages) and a copy of the device statistics block, every
// interval.  The sampler's kernel needs one block of 256 threads per 64 KiB
// of bitmap and fits beside a persistent batch kernel (which leaves registers
// and shared memory free on every SM), so samples are taken while the pool's
// own kernels run.  Samples are timestamped from the monitor's start.
#include <algorithm>
#include <chrono>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "internal.cuh"

namespace {

using Clock = std::chrono::steady_clock;

struct HostBlock {
    unsigned long long used;
    pbm::DevStats stats;
};

__global__ void __launch_bounds__(256) k_monitor_popcount(const unsigned long long* words, uint32_t n_words64,
                                                          unsigned long long* out) {
    unsigned long long c = 0;
    for (uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; w < n_words64; w += (uint64_t)gridDim.x * blockDim.x)
        c += (unsigned long long)__popcll(__ldcg(words + w));
    pbm::block_add_counters<1>({c}, {out});
}

}  // namespace

struct pbm_monitor {
    pbm_pool* pool = nullptr;
    int device = 0;
    uint32_t interval_us = 0;
    uint32_t max_samples = 0;
    cudaStream_t stream = nullptr;
    unsigned long long* d_count = nullptr;
    HostBlock* h_block = nullptr;   // pinned
    std::vector<pbm_monitor_sample> samples;
    std::mutex mu;
    std::thread th;
    std::atomic<bool> stop{false};
    std::atomic<int> status{PBM_OK};
    Clock::time_point t0;
};

static void monitor_loop(pbm_monitor* m) {
    if (cudaSetDevice(m->device) != cudaSuccess) {
        m->status = PBM_ERR_CUDA;
        return;
    }
    const uint32_t nw64 = m->pool->view.n_words64;
    const int blocks = (int)std::max<uint32_t>(1u, (nw64 + 256u * 64u - 1u) / (256u * 64u));
    while (!m->stop.load()) {
        bool ok = cudaMemsetAsync(m->d_count, 0, sizeof(unsigned long long), m->stream) == cudaSuccess;
        if (ok) {
            k_monitor_popcount<<<blocks, 256, 0, m->stream>>>(
                reinterpret_cast<const unsigned long long*>(m->pool->d_words), nw64, m->d_count);
            ok = cudaGetLastError() == cudaSuccess;
        }
        ok = ok && cudaMemcpyAsync(&m->h_block->used, m->d_count, sizeof(unsigned long long),
                                   cudaMemcpyDeviceToHost, m->stream) == cudaSuccess;
        ok = ok && cudaMemcpyAsync(&m->h_block->stats, m->pool->d_stats, sizeof(pbm::DevStats),
                                   cudaMemcpyDeviceToHost, m->stream) == cudaSuccess;
        ok = ok && cudaStreamSynchronize(m->stream) == cudaSuccess;
        if (!ok) {
            cudaGetLastError();
            m->status = PBM_ERR_CUDA;
            return;
        }
        pbm_monitor_sample smp{};
        smp.t_s = std::chrono::duration<double>(Clock::now() - m->t0).count();
        smp.used_pages = m->h_block->used - m->pool->padding_bits;
        smp.free_fraction = 1.0 - (double)smp.used_pages / (double)m->pool->n_pages;
        smp.stats.successes = m->h_block->stats.successes;
        smp.stats.failures = m->h_block->stats.failures;
        smp.stats.steps = m->h_block->stats.steps;
        smp.stats.frees = m->h_block->stats.frees;
        {
            std::lock_guard<std::mutex> lk(m->mu);
            m->samples.push_back(smp);
            if (m->samples.size() >= m->max_samples) return;
        }
        std::this_thread::sleep_for(std::chrono::microseconds(m->interval_us));
    }
}

extern "C" {

int pbm_monitor_start(pbm_pool* pool, uint32_t interval_us, uint32_t max_samples, pbm_monitor** out) {
    PBM_ON_POOL_DEVICE(pool);
    if (!pool || !out || max_samples == 0) return PBM_ERR_INVALID;
    *out = nullptr;
    pbm_monitor* m = new (std::nothrow) pbm_monitor();
    if (!m) return PBM_ERR_NOMEM;
    m->pool = pool;
    m->interval_us = interval_us;
    m->max_samples = max_samples;
    bool ok = cudaGetDevice(&m->device) == cudaSuccess &&
              cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) == cudaSuccess &&
              cudaMalloc(&m->d_count, sizeof(unsigned long long)) == cudaSuccess &&
              cudaMallocHost(&m->h_block, sizeof(HostBlock)) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        if (m->stream) cudaStreamDestroy(m->stream);
        cudaFree(m->d_count);
        cudaFreeHost(m->h_block);
        delete m;
        return PBM_ERR_NOMEM;
    }
    try {
        m->samples.reserve(max_samples);
        m->t0 = Clock::now();
        m->th = std::thread(monitor_loop, m);
    } catch (...) {
        cudaStreamDestroy(m->stream);
        cudaFree(m->d_count);
        cudaFreeHost(m->h_block);
        delete m;
        return PBM_ERR_NOMEM;
    }
    *out = m;
    return PBM_OK;
}

int pbm_monitor_samples(pbm_monitor* m, pbm_monitor_sample* h_out, uint32_t max_out, uint32_t* h_n) {
    if (!m || !h_n || (max_out && !h_out)) return PBM_ERR_INVALID;
    std::lock_guard<std::mutex> lk(m->mu);
    const uint32_t n = (uint32_t)m->samples.size();
    const uint32_t k = n < max_out ? n : max_out;
    for (uint32_t i = 0; i < k; ++i) h_out[i] = m->samples[i];
    *h_n = n;
    return m->status.load();
}

int pbm_monitor_stop(pbm_monitor* m) {
    if (!m) return PBM_ERR_INVALID;
    m->stop = true;
    if (m->th.joinable()) m->th.join();
    const int rc = m->status.load();
    cudaStreamDestroy(m->stream);
    cudaFree(m->d_count);
    cudaFreeHost(m->h_block);
    delete m;
    return rc;
}

}  // extern "C"
