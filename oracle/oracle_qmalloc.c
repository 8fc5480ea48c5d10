/* oracle_qmalloc.c -- sequential replay of the queue-based size classes
 * (TEST INFRASTRUCTURE ONLY).
 *
 * Restates the product's queue backend (pbm/pbm_qmalloc.cuh): per class
 * (16 B .. 64 KiB) a FIFO ring of free block handles (byte offset / 16).
 * For a group of up to 32 lanes: the lanes of each class, in lane order,
 * take blocks from the head of the class's ring; the lanes the ring cannot
 * serve are refill lanes: refill lane i takes block i % b of chunk i / b,
 * where a chunk (one page below a page-sized class, one block above) holding
 * b blocks is carved with the spanning walk by refill lane (i / b) * b, in
 * lane order over all classes; each carver enqueues its chunk's blocks that
 * no refill lane takes.  A free enqueues the block at the tail of its
 * class's ring; a full ring drops it.  One GPU warp with the carving
 * serialised must reproduce these offsets and the bitmap.  The queue idea
 * follows the page queues of the allocator the reference vendors as its
 * comparator (source/Ouroboros/include/device/queues/page/PageQueueVL_impl.cuh). */
#include "pbm_oracle.h"

#include <stdlib.h>
#include <string.h>

#define QCLASSES 13
#define QCONT 0x80u

static int q_class(uint64_t size) {
    if (size == 0 || size > (1ull << 16)) return -1;
    int c = 0;
    while ((1ull << (4 + c)) < size) ++c;
    return c;
}

static uint32_t chunk_bytes(const orc_qmalloc_t *q, int c) {
    const uint32_t b = 1u << (4 + c), page = 1u << q->page_shift;
    return b > page ? b : page;
}

int orc_qmalloc_init(orc_qmalloc_t *q, uint32_t *words, uint32_t n_pages, uint32_t page_shift, uint32_t cap) {
    memset(q, 0, sizeof(*q));
    q->words = words;
    q->n_pages = n_pages;
    q->page_shift = page_shift;
    q->cap = cap;
    q->class_of = (uint8_t *)calloc(n_pages, 1);
    q->ring = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)QCLASSES * cap);
    if (!q->class_of || !q->ring) return -1;
    memset(q->ring, 0xff, sizeof(uint32_t) * (size_t)QCLASSES * cap);
    for (int c = 0; c < QCLASSES; ++c) q->space[c] = cap;
    return 0;
}

void orc_qmalloc_destroy(orc_qmalloc_t *q) {
    free(q->class_of);
    free(q->ring);
    q->class_of = NULL;
    q->ring = NULL;
}

static void enqueue_run(orc_qmalloc_t *q, int c, uint32_t first, uint32_t stride, uint32_t n) {
    if (n == 0) return;
    int64_t got = q->space[c] <= 0 ? 0 : (q->space[c] < (int64_t)n ? q->space[c] : (int64_t)n);
    q->space[c] -= got;
    q->overflow += n - (uint64_t)got;
    for (int64_t i = 0; i < got; ++i)
        q->ring[(size_t)c * q->cap + ((q->tail[c] + (uint64_t)i) & (q->cap - 1u))] = first + (uint32_t)i * stride;
    q->tail[c] += (uint64_t)got;
    q->avail[c] += got;
}

void orc_qmalloc_group(orc_qmalloc_t *q, const uint64_t *sizes, int lanes, const int32_t *seed_own,
                       uint32_t max_steps, int64_t *offsets, int32_t *steps) {
    int cls[32], rank[32], k_of[32];
    uint32_t got_of[32];
    for (int l = 0; l < lanes; ++l) {
        cls[l] = q_class(sizes[l]);
        offsets[l] = -1;
        steps[l] = 0;
    }
    for (int l = 0; l < lanes; ++l) {
        rank[l] = 0;
        k_of[l] = 0;
        if (cls[l] < 0) continue;
        for (int j = 0; j < lanes; ++j) {
            if (cls[j] != cls[l]) continue;
            ++k_of[l];
            if (j < l) ++rank[l];
        }
    }
    /* 1. blocks from the rings: the first lane of each class reserves */
    for (int l = 0; l < lanes; ++l) got_of[l] = 0;
    for (int l = 0; l < lanes; ++l) {
        if (cls[l] < 0 || rank[l] != 0) continue;
        const int c = cls[l];
        const int64_t k = k_of[l];
        const int64_t got = q->avail[c] <= 0 ? 0 : (q->avail[c] < k ? q->avail[c] : k);
        q->avail[c] -= got;
        const uint64_t h0 = q->head[c];
        q->head[c] += (uint64_t)got;
        for (int j = 0; j < lanes; ++j) {
            if (cls[j] != c) continue;
            got_of[j] = (uint32_t)got;
            if ((int64_t)rank[j] < got) {
                uint32_t *slot = &q->ring[(size_t)c * q->cap + ((h0 + (uint64_t)rank[j]) & (q->cap - 1u))];
                offsets[j] = (int64_t)(*slot) * 16;
                *slot = 0xffffffffu;
            }
        }
        q->space[c] += got;
    }
    /* 2. refill lanes: carvers in lane order, then every refill lane takes its block */
    int32_t chunk_of[32];
    for (int l = 0; l < lanes; ++l) chunk_of[l] = -1;
    for (int l = 0; l < lanes; ++l) {
        if (cls[l] < 0 || (uint32_t)rank[l] < got_of[l]) continue;
        const int c = cls[l];
        const uint32_t b = chunk_bytes(q, c) >> (4 + c);
        const uint32_t ri = (uint32_t)rank[l] - got_of[l], r_total = (uint32_t)k_of[l] - got_of[l];
        if (ri % b != 0) continue;
        const uint32_t npages = chunk_bytes(q, c) >> q->page_shift;
        int32_t s = 0;
        const int32_t ch = orc_walk_span(q->words, q->n_pages, npages, seed_own[l], max_steps, &s);
        steps[l] = s;
        chunk_of[l] = ch;
        if (ch < 0) continue;
        q->class_of[ch] = (uint8_t)(c + 1);
        for (uint32_t p = 1; p < npages; ++p) q->class_of[ch + (int32_t)p] = (uint8_t)(QCONT | (uint32_t)(c + 1));
        ++q->chunks;
        const uint32_t bytes = 1u << (4 + c);
        const uint32_t first = (uint32_t)(((uint64_t)(uint32_t)ch << q->page_shift) >> 4);
        const uint32_t users = r_total - ri < b ? r_total - ri : b;
        enqueue_run(q, c, first + users * (bytes >> 4), bytes >> 4, b - users);
    }
    for (int l = 0; l < lanes; ++l) {
        if (cls[l] < 0 || (uint32_t)rank[l] < got_of[l]) continue;
        const int c = cls[l];
        const uint32_t b = chunk_bytes(q, c) >> (4 + c);
        const uint32_t ri = (uint32_t)rank[l] - got_of[l];
        const uint32_t carver_ri = (ri / b) * b;
        int carver = -1;
        for (int j = 0; j < lanes; ++j)
            if (cls[j] == c && (uint32_t)rank[j] >= got_of[j] && (uint32_t)rank[j] - got_of[j] == carver_ri) carver = j;
        if (carver >= 0 && chunk_of[carver] >= 0)
            offsets[l] = ((int64_t)chunk_of[carver] << q->page_shift) + (int64_t)(ri % b) * (1 << (4 + c));
    }
}

void orc_qmalloc_free_group(orc_qmalloc_t *q, const int64_t *offsets, int lanes, int32_t *ok) {
    int cls[32];
    for (int l = 0; l < lanes; ++l) {
        cls[l] = -1;
        ok[l] = 1;
        const int64_t off = offsets[l];
        if (off < 0) continue;
        if ((uint64_t)off >= ((uint64_t)q->n_pages << q->page_shift) || (off & 15)) { ok[l] = 0; ++q->bad_frees; continue; }
        const uint8_t mark = q->class_of[off >> q->page_shift];
        const int c = (int)(mark & 0x7fu) - 1;
        const uint32_t page = 1u << q->page_shift;
        const uint64_t align = c >= 0 ? ((1u << (4 + c)) < page ? (1u << (4 + c)) : page) : 1;
        if (c < 0 || (mark & QCONT) || (off & (int64_t)(align - 1))) { ok[l] = 0; ++q->bad_frees; continue; }
        cls[l] = c;
    }
    for (int c = 0; c < QCLASSES; ++c) {
        int64_t k = 0;
        for (int l = 0; l < lanes; ++l) k += cls[l] == c;
        if (!k) continue;
        const int64_t got = q->space[c] <= 0 ? 0 : (q->space[c] < k ? q->space[c] : k);
        q->space[c] -= got;
        q->overflow += (uint64_t)(k - got);
        int64_t r = 0;
        for (int l = 0; l < lanes; ++l) {
            if (cls[l] != c) continue;
            if (r < got) q->ring[(size_t)c * q->cap + ((q->tail[c] + (uint64_t)r) & (q->cap - 1u))] = (uint32_t)(offsets[l] >> 4);
            ++r;
        }
        q->tail[c] += (uint64_t)got;
        q->avail[c] += got;
    }
}
