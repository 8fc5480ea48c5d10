/* oracle_malloc.c -- sequential replay of the size-classed malloc
 * (TEST INFRASTRUCTURE ONLY).
 *
 * Restates the product's malloc over the page bitmap: sizes rounded up to
 * power-of-two classes (16 B .. 64 KiB); the sub-page requests of a group of
 * 32 share one run, packed largest class first; page-sized and larger
 * requests take their own run, in lane order; every run keeps a live-block
 * count and the last free releases it.  The idea follows the reference's
 * mallocRW / freeRW (source/RWMalloc.cuh:299-334), whose non-leader blocks
 * are never released.  One GPU warp running the same group with its large
 * claims serialised must reproduce these offsets, steps and the bitmap. */
#include "pbm_oracle.h"

#include <string.h>

static int malloc_class(uint64_t size) {
    if (size == 0 || size > (1ull << 16)) return -1;
    int c = 0;
    while ((1ull << (4 + c)) < size) ++c;
    return c;
}

static void mark_run(orc_malloc_t *m, int32_t start, uint32_t n, int32_t blocks) {
    for (uint32_t k = 0; k < n; ++k) m->start_of[start + (int32_t)k] = start;
    m->len_of[start] = (uint8_t)n;
    m->live[start] = blocks;
}

void orc_malloc_group(orc_malloc_t *m, const uint64_t *sizes, int lanes, int32_t seed_small,
                      const int32_t *seed_own, uint32_t max_steps, int64_t *offsets, int32_t *steps) {
    const uint32_t page = 1u << m->page_shift;
    const int max_small = (int)m->page_shift - 1 - 4;
    int cls[32];
    uint32_t bytes[32], off[32];
    int small[32], large[32];
    for (int l = 0; l < lanes; ++l) {
        cls[l] = malloc_class(sizes[l]);
        bytes[l] = cls[l] >= 0 ? (1u << (4 + cls[l])) : 0u;
        small[l] = cls[l] >= 0 && bytes[l] < page;
        large[l] = cls[l] >= 0 && bytes[l] >= page;
        offsets[l] = -1;
        steps[l] = 0;
        off[l] = 0;
    }
    uint32_t total = 0;
    for (int c = max_small; c >= 0; --c)
        for (int l = 0; l < lanes; ++l)
            if (small[l] && cls[l] == c) { off[l] = total; total += 1u << (4 + c); }
    int leader = -1, n_small = 0;
    for (int l = 0; l < lanes; ++l) if (small[l]) { if (leader < 0) leader = l; ++n_small; }
    if (leader >= 0) {
        const uint32_t n = (total + page - 1u) >> m->page_shift;
        int32_t s = 0;
        int32_t start = orc_walk_span(m->words, m->n_pages, n, seed_small, max_steps, &s);
        steps[leader] += s;
        if (start >= 0) {
            mark_run(m, start, n, n_small);
            for (int l = 0; l < lanes; ++l)
                if (small[l]) offsets[l] = ((int64_t)start << m->page_shift) + off[l];
        }
    }
    for (int l = 0; l < lanes; ++l) {
        if (!large[l]) continue;
        const uint32_t n = bytes[l] >> m->page_shift;
        int32_t s = 0;
        int32_t start = orc_walk_span(m->words, m->n_pages, n, seed_own[l], max_steps, &s);
        steps[l] += s;
        if (start >= 0) {
            mark_run(m, start, n, 1);
            offsets[l] = (int64_t)start << m->page_shift;
        }
    }
}

int orc_malloc_free(orc_malloc_t *m, int64_t offset) {
    if (offset < 0 || (uint64_t)offset >= ((uint64_t)m->n_pages << m->page_shift)) return 0;
    int32_t pg = (int32_t)(offset >> m->page_shift);
    int32_t run = m->start_of[pg];
    if (run < 0 || m->live[run] <= 0) return 0;
    if (--m->live[run] == 0) orc_free_run(m->words, run, m->len_of[run]);
    return 1;
}
