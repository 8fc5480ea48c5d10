/* oracle_bufmgr.c -- single-thread replay of the CLOCK buffer manager
 * (TEST INFRASTRUCTURE ONLY).
 *
 * The reference has no buffer manager (its SingleClock / DistClock arms,
 * parallelPage.cu:491-509 and 571-592, sweep a free map), so this replay
 * restates the semantics the product defines: a fetch of a resident page
 * pins it and sets its reference bit (hit); otherwise the hand sweeps frames
 * -- pinned ones are skipped, referenced ones lose their bit (second
 * chance) -- and the first unpinned unreferenced frame is taken, its old
 * page unmapped (eviction) and the new one mapped (miss).  One GPU thread
 * running the same rounds must reproduce every frame id and counter. */
#include "pbm_oracle.h"

#include <stdlib.h>
#include <string.h>

#define EMPTY_PAGE 0xffffffffu

void orc_bm_init(orc_bm_t *b, uint32_t n_logical, uint32_t n_frames, uint32_t max_sweep,
                 uint32_t n_arms, int dist) {
    memset(b, 0, sizeof(*b));
    b->n_logical = n_logical;
    b->n_frames = n_frames;
    b->max_sweep = max_sweep ? max_sweep : 2u * n_frames + 64u;
    b->n_arms = n_arms ? n_arms : 1u;
    b->dist = dist;
    b->page_table = (int32_t *)malloc(sizeof(int32_t) * n_logical);
    b->frame_state = (uint64_t *)malloc(sizeof(uint64_t) * n_frames);
    b->ref = (uint8_t *)calloc(n_frames, 1);
    b->arms = (uint32_t *)malloc(sizeof(uint32_t) * b->n_arms);
    for (uint32_t p = 0; p < n_logical; ++p) b->page_table[p] = -1;
    for (uint32_t f = 0; f < n_frames; ++f) b->frame_state[f] = (uint64_t)EMPTY_PAGE << 32;
    for (uint32_t a = 0; a < b->n_arms; ++a) b->arms[a] = (uint32_t)(((uint64_t)a * n_frames) / b->n_arms);
}

void orc_bm_free(orc_bm_t *b) {
    free(b->page_table);
    free(b->frame_state);
    free(b->ref);
    free(b->arms);
    memset(b, 0, sizeof(*b));
}

static uint32_t next_frame(orc_bm_t *b, uint32_t *arm) {
    if (!b->dist) return (uint32_t)((b->hand++) % b->n_frames);
    uint32_t a = *arm;
    uint32_t f = a >= b->n_frames ? a - b->n_frames : a;
    *arm = f + 1u;
    return f;
}

int32_t orc_bm_fetch(orc_bm_t *b, uint32_t page, uint32_t slot) {
    int32_t f = b->page_table[page];
    if (f >= 0) {
        b->frame_state[f] += 1u;
        b->ref[f] = 1;
        b->hits++;
        return f;
    }
    uint32_t arm = b->dist ? b->arms[slot] : 0u;
    int32_t h = -1;
    for (uint32_t i = 0; i < b->max_sweep; ++i) {
        uint32_t fr = next_frame(b, &arm);
        uint64_t s = b->frame_state[fr];
        if ((uint32_t)s != 0u) continue;
        if (b->ref[fr]) { b->ref[fr] = 0; continue; }
        b->frame_state[fr] = ((uint64_t)page << 32) | 1u;
        uint32_t old = (uint32_t)(s >> 32);
        if (old != EMPTY_PAGE) {
            b->page_table[old] = -1;
            b->evictions++;
        }
        h = (int32_t)fr;
        break;
    }
    if (b->dist) b->arms[slot] = arm;
    if (h < 0) {
        b->failures++;
        return -1;
    }
    b->ref[h] = 1;
    b->page_table[page] = h;
    b->misses++;
    return h;
}

void orc_bm_unpin(orc_bm_t *b, int32_t f) {
    if (f < 0 || (uint32_t)f >= b->n_frames) return;
    if ((uint32_t)b->frame_state[f] == 0u) { b->bad_unpins++; return; }
    b->frame_state[f] -= 1u;
    b->unpins++;
}

void orc_bm_round(orc_bm_t *b, const int32_t *frames_of, const int32_t *release_idx, uint32_t n_release,
                  const int32_t *pages, uint32_t n, uint32_t slot0, int32_t *frames_out) {
    for (uint32_t j = 0; j < n_release; ++j) orc_bm_unpin(b, frames_of[release_idx[j]]);
    for (uint32_t i = 0; i < n; ++i) {
        int32_t p = pages[i];
        frames_out[i] = (p >= 0 && (uint32_t)p < b->n_logical)
                            ? orc_bm_fetch(b, (uint32_t)p, (slot0 + i) % b->n_arms)
                            : -1;
    }
}
