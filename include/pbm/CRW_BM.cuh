// Drop-in for source/CRW_BM.cuh: clustered walk.  Each global thread id
// keeps the last page it obtained (slot tid % PBM_DROPIN_SLOTS) and resumes
// in that word; otherwise random word-probe jumps.  steps = claim attempts.
#pragma once
#include "pbm/header_only_common.cuh"

/* getPage(int* step_count): CRW_BM.cuh:75-142 */
__device__ inline int getPage(int* step_count = 0) {
    const pbm::dropin::DeviceState& d = pbm_tu_state;
    if (!d.valid) return -1;
    int32_t* cur = d.cursors + (pbm::dropin::global_tid() % d.max_slots);
    int32_t c = *cur;
    int id = pbm::walk_crw(d.view, &c, pbm::dropin::call_seed(), PBM_DROPIN_MAX_STEPS, step_count);
    *cur = c;
    return id;
}
__device__ inline void* getPagePtr() {
    int id = getPage();
    return id >= 0 ? pageAddress(id) : nullptr;
}
/* freePage(pageID): CRW_BM.cuh:152-156 */
__device__ inline void freePage(int pageID) { pbm::dropin::free_checked(pbm_tu_state, pageID); }
