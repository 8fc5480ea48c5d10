// Drop-in for source/CollabRW_BM.cuh: warp-collaborative walk over the lanes
// that call getPage together (__activemask()).  Exactly the needed bits are
// claimed, one atomicOr per word, so nothing is written back; steps = warp
// iterations, equal for all calling lanes.  Blocks must be 1-D with at most
// 1024 threads (4 KB of shared memory per block, as in the reference).
#pragma once
#include "pbm/header_only_common.cuh"

/* getPage(int* step_count, bool collectWarpData): CollabRW_BM.cuh:114-160.
 * collectWarpData prints the warp's step count from its first calling lane
 * (the reference prints pages found per warp step). */
__device__ inline int getPage(int* step_count = 0, bool collectWarpData = false) {
    int s = 0;
    int id = pbm::dropin::collab_get(pbm_tu_state, &s);
    if (step_count) *step_count = s;
    if (collectWarpData && (threadIdx.x & 31u) == (unsigned)(__ffs((int)__activemask()) - 1)) printf("%d\n", s);
    return id;
}
__device__ inline void* getPagePtr() {
    int id = getPage();
    return id >= 0 ? pageAddress(id) : nullptr;
}
/* freePage(pageID): CollabRW_BM.cuh:73-77 */
__device__ inline void freePage(int pageID) { pbm::dropin::free_checked(pbm_tu_state, pageID); }
