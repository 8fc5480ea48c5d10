// autotune.cu -- picks the batch kernel configuration for a pool's occupancy.
//
// The sweep covers the walk (per-thread page probe, per-thread word probe,
// warp-collaborative), the collaboration width (8 / 16 / 32 lanes, or 64:
// 32 lanes serving two requests each), 32- vs
// 64-bit bitmap words, the walk stride between a group's lanes, and blocks
// per SM (occupancy-limited, or register-capped at kCappedBlocks), and merged
// frees.  Every candidate runs the caller's own batch of swap requests through
// the persistent kernel once untimed and then `reps` times, each timed alone
// with CUDA events after the L2 is flushed (a 256 MiB write, twice the L2), as
// a batch that arrives after other work would find it; the median time
// ranks the candidate, the mean breaks ties between equal medians (event
// times are quantised, so close candidates often share a median), and a
// stable sort keeps the candidate order where both tie.  A swap frees one page for every page it takes, so the
// pool stays in its occupancy band while it is tuned.  The
// caller tunes once per band (e.g. after prefilling to 50/75/90/95%) and keeps
// the winning configuration per band.
#include <algorithm>
#include <vector>

#include "internal.cuh"

using namespace pbm;

namespace {

std::vector<pbm_walk_config> candidates(uint32_t max_steps) {
    std::vector<pbm_walk_config> out;
    auto base = [&]() {
        pbm_walk_config c{};
        c.max_steps = max_steps;
        c.block_size = 256;
        c.free_merge = 0;
        c.stride = 1;
        c.word_bits = 32;
        c.collab_width = 32;
        return c;
    };
    for (int bps : {0, kCappedBlocks}) {
        pbm_walk_config c = base();
        c.strategy = PBM_RANDOM_WALK;
        c.blocks_per_sm = bps;
        out.push_back(c);
        for (int wb : {32, 64}) {
            c = base();
            c.strategy = PBM_RANDOM_WALK_BM;
            c.word_bits = wb;
            c.blocks_per_sm = bps;
            out.push_back(c);
        }
        for (int wb : {32, 64})
            for (int W : {8, 16, 32, 64})
                for (uint32_t stride : {1u, 33u}) {
                    c = base();
                    c.strategy = PBM_COLLAB_RW_BM;
                    c.word_bits = wb;
                    c.collab_width = W;
                    c.stride = stride;
                    c.blocks_per_sm = bps;
                    out.push_back(c);
                }
    }
    // the free-merge knob on the default collaborative configuration
    for (int bps : {0, kCappedBlocks}) {
        pbm_walk_config c = base();
        c.strategy = PBM_COLLAB_RW_BM;
        c.blocks_per_sm = bps;
        c.free_merge = 1;
        out.push_back(c);
    }
    return out;
}

}  // namespace

extern "C" int pbm_autotune(pbm_pool* pool, const pbm_group* d_groups, uint32_t n_groups, uint64_t requests,
                            int32_t* d_arena, uint64_t arena_len, uint32_t seed, int reps, uint32_t max_steps,
                            pbm_tune_result* h_out, uint32_t max_out, uint32_t* h_n_out, void* stream) {
    PBM_ON_POOL_DEVICE(pool);
    if (!pool || !d_groups || !n_groups || !d_arena || !arena_len || reps < 1 || !h_out || !max_out || !h_n_out)
        return PBM_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    std::vector<pbm_walk_config> cands = candidates(max_steps ? max_steps : kDefaultMaxSteps);
    std::vector<pbm_tune_result> res;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    void* flush = nullptr;
    const size_t flush_bytes = size_t(256) << 20;
    if (cudaMalloc(&flush, flush_bytes) != cudaSuccess) {   // tune without flushes rather than fail
        cudaGetLastError();
        flush = nullptr;
    }
    auto cleanup = [&]() {
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        if (flush) cudaFree(flush);
    };
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        cudaGetLastError();
        cleanup();
        return PBM_ERR_CUDA;
    }
    uint32_t sd = seed;
    std::vector<float> times((size_t)reps);
    int rc = PBM_OK;
    for (const pbm_walk_config& c : cands) {
        // one untimed launch (first-use costs), then `reps` launches, each timed after an L2 flush
        rc = pbm_batch_launch(pool, &c, d_groups, nullptr, n_groups, d_arena, arena_len, sd++, nullptr,
                              PBM_LAUNCH_PERSISTENT, s);
        if (rc == PBM_ERR_UNSUPPORTED) { rc = PBM_OK; continue; }
        for (int r = 0; r < reps && rc == PBM_OK; ++r) {
            if (flush && cudaMemsetAsync(flush, r & 0xff, flush_bytes, s) != cudaSuccess) rc = PBM_ERR_CUDA;
            if (!rc && cudaEventRecord(e0, s) != cudaSuccess) rc = PBM_ERR_CUDA;
            if (!rc) rc = pbm_batch_launch(pool, &c, d_groups, nullptr, n_groups, d_arena, arena_len, sd++, nullptr,
                                           PBM_LAUNCH_PERSISTENT, s);
            if (!rc && (cudaEventRecord(e1, s) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                        cudaEventElapsedTime(&times[(size_t)r], e0, e1) != cudaSuccess))
                rc = PBM_ERR_CUDA;
        }
        if (rc) break;
        double sum = 0.0;
        for (float x : times) sum += x;
        std::sort(times.begin(), times.end());
        const float ms = times[(size_t)reps / 2];
        pbm_tune_result t{};
        t.cfg = c;
        t.ms_per_batch = ms;
        t.ms_mean = (float)(sum / reps);
        t.ops_per_s = ms > 0.f ? 2.0 * (double)requests / (ms * 1e-3) : 0.0;
        res.push_back(t);
    }
    if (rc == PBM_ERR_CUDA) cudaGetLastError();
    cleanup();
    if (rc) return rc;
    std::stable_sort(res.begin(), res.end(), [](const pbm_tune_result& a, const pbm_tune_result& b) {
        if (a.ms_per_batch != b.ms_per_batch) return a.ms_per_batch < b.ms_per_batch;
        return a.ms_mean < b.ms_mean;
    });
    const uint32_t n = (uint32_t)std::min<size_t>(res.size(), max_out);
    for (uint32_t i = 0; i < n; ++i) h_out[i] = res[i];
    *h_n_out = n;
    return PBM_OK;
}
