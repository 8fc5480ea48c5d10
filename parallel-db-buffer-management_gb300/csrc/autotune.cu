// autotune.cu -- picks the batch kernel configuration for a pool's occupancy.
//
// The sweep covers the walk (per-thread page probe, per-thread word probe,
// warp-collaborative), the collaboration width (8 / 16 / 32 lanes), 32- vs
// 64-bit bitmap words, the walk stride between a group's lanes, and blocks
// per SM (occupancy-limited, or register-capped at 6), and merged frees.  Every candidate
// runs the caller's own batch of swap requests through the persistent kernel
// `reps` times, timed with CUDA events; a swap frees one page for every page
// it takes, so the pool stays in its occupancy band while it is tuned.  The
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
        c.free_merge = 1;
        c.stride = 1;
        c.word_bits = 32;
        c.collab_width = 32;
        return c;
    };
    for (int bps : {0, 6}) {
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
            for (int W : {8, 16, 32})
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
    pbm_walk_config c = base();
    c.strategy = PBM_COLLAB_RW_BM;
    c.free_merge = 0;
    out.push_back(c);
    return out;
}

}  // namespace

extern "C" int pbm_autotune(pbm_pool* pool, const pbm_group* d_groups, uint32_t n_groups, uint64_t requests,
                            int32_t* d_arena, uint64_t arena_len, uint32_t seed, int reps, uint32_t max_steps,
                            pbm_tune_result* h_out, uint32_t max_out, uint32_t* h_n_out, void* stream) {
    if (!pool || !d_groups || !n_groups || !d_arena || !arena_len || reps < 1 || !h_out || !max_out || !h_n_out)
        return PBM_ERR_INVALID;
    cudaStream_t s = (cudaStream_t)stream;
    std::vector<pbm_walk_config> cands = candidates(max_steps ? max_steps : kDefaultMaxSteps);
    std::vector<pbm_tune_result> res;
    cudaEvent_t e0, e1;
    PBM_CUDA_TRY(cudaEventCreate(&e0));
    PBM_CUDA_TRY(cudaEventCreate(&e1));
    uint32_t sd = seed;
    for (const pbm_walk_config& c : cands) {
        // one untimed launch (first-use costs), then `reps` timed launches
        int rc = pbm_batch_launch(pool, &c, d_groups, nullptr, n_groups, d_arena, arena_len, sd++, nullptr,
                                  PBM_LAUNCH_PERSISTENT, s);
        if (rc == PBM_ERR_UNSUPPORTED) continue;
        if (rc) { cudaEventDestroy(e0); cudaEventDestroy(e1); return rc; }
        PBM_CUDA_TRY(cudaEventRecord(e0, s));
        for (int r = 0; r < reps && rc == PBM_OK; ++r)
            rc = pbm_batch_launch(pool, &c, d_groups, nullptr, n_groups, d_arena, arena_len, sd++, nullptr,
                                  PBM_LAUNCH_PERSISTENT, s);
        if (rc) { cudaEventDestroy(e0); cudaEventDestroy(e1); return rc; }
        PBM_CUDA_TRY(cudaEventRecord(e1, s));
        PBM_CUDA_TRY(cudaEventSynchronize(e1));
        float ms = 0.f;
        PBM_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
        pbm_tune_result t{};
        t.cfg = c;
        t.ms_per_batch = ms / (float)reps;
        t.ops_per_s = ms > 0.f ? 2.0 * (double)requests * reps / (ms * 1e-3) : 0.0;
        res.push_back(t);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    std::sort(res.begin(), res.end(),
              [](const pbm_tune_result& a, const pbm_tune_result& b) { return a.ops_per_s > b.ops_per_s; });
    const uint32_t n = (uint32_t)std::min<size_t>(res.size(), max_out);
    for (uint32_t i = 0; i < n; ++i) h_out[i] = res[i];
    *h_n_out = n;
    return PBM_OK;
}
