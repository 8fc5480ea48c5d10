// Drop-in for source/RandomWalkBasic.cuh: per-thread page-probe random walk.
// getPage probes random pages until it claims one (steps = probes); the
// reference's int-per-page map is a bitmap here.
#pragma once
#include "pbm/header_only_common.cuh"

/* getPage(int* step_count): RandomWalkBasic.cuh:54-74 (-1 when the step bound runs out) */
__device__ inline int getPage(int* step_count = 0) {
    if (!pbm_tu_state.valid) return -1;
    return pbm::walk_page(pbm_tu_state.view, pbm::dropin::call_seed(), PBM_DROPIN_MAX_STEPS, step_count);
}
/* getPagePtr(): RandomWalkBasic.cuh:76-79 */
__device__ inline void* getPagePtr() {
    int id = getPage();
    return id >= 0 ? pageAddress(id) : nullptr;
}
/* freePage(pageID): RandomWalkBasic.cuh:82-84 */
__device__ inline void freePage(int pageID) { pbm::dropin::free_checked(pbm_tu_state, pageID); }
