// Drop-in for source/RandomWalkBasic_BM.cuh: per-thread word-probe walk over
// a 32-bit bitmap (steps = random jumps).  Returns the claimed page's id;
// the reference's `groupID<<5 + bitPosition` expression is not reproduced.
#pragma once
#include "pbm/header_only_common.cuh"

/* getPage(int* step_count): RandomWalkBasic_BM.cuh:60-89 */
__device__ inline int getPage(int* step_count = 0) {
    if (!pbm_tu_state.valid) return -1;
    return pbm::walk_word<uint32_t>(pbm_tu_state.view, pbm::dropin::call_seed(), PBM_DROPIN_MAX_STEPS,
                                    step_count);
}
__device__ inline void* getPagePtr() {
    int id = getPage();
    return id >= 0 ? pageAddress(id) : nullptr;
}
/* freePage(pageID): RandomWalkBasic_BM.cuh:98-102 */
__device__ inline void freePage(int pageID) { pbm::dropin::free_checked(pbm_tu_state, pageID); }
