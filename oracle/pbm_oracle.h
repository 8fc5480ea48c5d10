/*
 * pbm_oracle.h -- CPU oracle for the GPU page/buffer manager.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product links, loads or calls
 * this code; only the tests, the smoke check and the CPU-baseline leg of the
 * benchmark do, and only as the checker (or as the timed CPU baseline).
 *
 * Two families of functions live here:
 *
 *   orc_ref_*   restatements of the reference's device routines, step for
 *               step, including their quirks (clock-derived seeds, the
 *               `groupID<<5 + bit` id expression, word grabbing with
 *               atomicExch).  They are pinned against outputs of the
 *               reference's own code, compiled for the GPU from its sources
 *               and run single-threaded / single-warp with a fixed clock
 *               (golden fixtures under tests/golden/).
 *
 *   orc_*       sequential replays of the product's algorithms (same LCG,
 *               same claim order, same step counting).  A single-thread or
 *               single-warp GPU launch of the product must reproduce them
 *               bit for bit: page ids, step counts and the final bitmap.
 *
 * Bitmaps are arrays of 32-bit words, bit b of word w <-> page 32*w+b,
 * bit set = page held.  Bits past the last page of the pool are kept set.
 */
#ifndef PBM_ORACLE_H
#define PBM_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ */
/* Primitives                                                          */
/* ------------------------------------------------------------------ */

/* One step of the reference LCG (source/RNG_LCG.cuh:9-12):
 * (1103515245*x + 12345) computed in signed 64-bit, C-truncating remainder
 * by 2^31, cast to int. */
int32_t orc_lcg(int32_t x);

/* Reference index mapping: (unsigned)x % n. */
uint32_t orc_idx_mod(int32_t x, uint32_t n);

/* Product index mapping: the LCG's 31 state bits scaled onto [0, n) by a
 * multiply-high, so the index comes from the well-mixed high bits. */
uint32_t orc_idx_hi(int32_t x, uint32_t n);

/* Product per-request seed: a mixed hash of (stream seed S, request r),
 * reduced to 31 bits so the LCG sequence stays non-negative. */
int32_t orc_seed(uint32_t S, uint32_t r);

/* Counter-based 64-bit hash used by the Bernoulli prefill. */
uint64_t orc_hash64(uint64_t seed, uint64_t ctr);

/* PTX-style shift semantics (shift amounts >= 32 give 0). */
uint32_t orc_shl32(uint32_t x, uint32_t n);

/* ------------------------------------------------------------------ */
/* Bitmaps                                                             */
/* ------------------------------------------------------------------ */

size_t orc_words_for(uint64_t n_pages, int word_bits);

/* Fill a bitmap with i.i.d. Bernoulli(occ) bits, one hash per page.
 * Bit for page p is set iff (hash64(seed, p) >> 11) < thresh53 where
 * thresh53 = (uint64_t)(occ * 2^53).  Padding bits are set. */
void orc_prefill_bernoulli(uint32_t *words, uint64_t n_pages, uint64_t thresh53, uint64_t seed);
uint64_t orc_thresh53(double occ);

/* Set the padding bits past n_pages (32-bit words). */
void orc_set_padding(uint32_t *words, uint64_t n_pages);

/* Number of held pages (padding bits excluded). */
uint64_t orc_used_pages(const uint32_t *words, uint64_t n_pages);

/* ------------------------------------------------------------------ */
/* Invariant checker                                                   */
/* ------------------------------------------------------------------ */

typedef struct {
    int64_t n_ok;          /* ids >= 0 */
    int64_t n_failed;      /* ids == -1 */
    int64_t n_out_of_range;
    int64_t n_duplicates;  /* ids returned to more than one requester */
    int64_t n_not_marked;  /* returned ids whose bit is clear */
    int64_t n_prefilled;   /* returned ids that were already held before */
    int64_t used_after;    /* popcount of the bitmap */
} orc_check_t;

/* Check the allocation invariants of ids[0..n) against the bitmap after the
 * allocation and the bitmap before it (may be NULL). */
void orc_check_alloc(const uint32_t *after, const uint32_t *before, uint64_t n_pages,
                     const int32_t *ids, int64_t n, orc_check_t *out);

/* ------------------------------------------------------------------ */
/* Product-mode sequential replays                                     */
/* ------------------------------------------------------------------ */

/* Per-thread page-probe walk (RandomWalkBasic semantics on a bitmap):
 * probe random pages until one is claimed.  Steps = probes. */
int32_t orc_walk_page(uint32_t *words, uint32_t n_pages, int32_t seed0,
                      uint32_t max_steps, int32_t *steps);

/* Per-thread word-probe walk (RandomWalkBasic_BM semantics): jump to a
 * random word, claim its lowest clear bits until one sticks.
 * Steps = random jumps.  word_bits = 32 or 64 (64-bit words are pairs of
 * 32-bit words, little-endian, bit b of 64-bit word w = page 64*w+b). */
int32_t orc_walk_word(uint32_t *words, uint32_t n_pages, int word_bits, int32_t seed0,
                      uint32_t max_steps, int32_t *steps);

/* Warp-collaborative walk over 32/64-bit words.
 * lanes: number of lanes in the collaborating group (1..32); need[i] = lane
 * i requests one page.  All lanes share one seed (seed0 of the group's
 * first lane).  Each iteration: jump to base = idx(seed, n_words); lane i
 * reads word (base + i*stride) mod n_words; the group claims exactly as many
 * clear bits as it still needs, lowest lanes and lowest bits first, with one
 * atomic OR per word; gained pages are handed to the needing lanes in lane
 * order.  Duplicate words within one iteration are read only by their lowest
 * lane.  steps[i] = iterations run by the group (same for all lanes).
 * ids[i] = page or -1. */
void orc_walk_collab(uint32_t *words, uint32_t n_pages, int word_bits, int lanes,
                     const uint8_t *need, int32_t seed0, uint32_t stride,
                     uint32_t max_steps, int32_t *ids, int32_t *steps);

/* Clustered walk (CRW_BM semantics): resume at the word of the last page
 * this slot obtained (next word when the last bit was the word's top bit),
 * claim lowest clear bits there; otherwise random word-probe walk.
 * cursor: last page of this slot or -1.  Steps = claim attempts. */
int32_t orc_walk_crw(uint32_t *words, uint32_t n_pages, int32_t *cursor, int32_t seed0,
                     uint32_t max_steps, int32_t *steps);

/* Single clock (parallelPage.cu getPageSingleClock semantics, with the
 * claim made by test-and-set): take arm position, arm++, claim if clear. */
int32_t orc_single_clock(uint32_t *words, uint32_t n_pages, uint64_t *arm,
                         uint32_t max_steps, int32_t *steps);

/* Distributed clock (getPageDistClock semantics): per-slot arm, linear
 * probe from the arm, arm moves past every probed page. */
int32_t orc_dist_clock(uint32_t *words, uint32_t n_pages, uint32_t *arm,
                       uint32_t max_steps, int32_t *steps);
/* Initial arm of a slot: idx(lcg(seed(S, slot)), n_pages). */
uint32_t orc_dist_clock_arm0(uint32_t S, uint32_t slot, uint32_t n_pages);

/* Contiguous run of n pages (1 <= n <= 32) inside one 32-bit word, by
 * word-probe walk; the lowest run start in the word is taken. */
int32_t orc_walk_run(uint32_t *words, uint32_t n_pages, uint32_t n, int32_t seed0,
                     uint32_t max_steps, int32_t *steps);

/* Contiguous run of n pages (1 <= n <= 65536) that may cross word
 * boundaries: per jump, scan from a random word for a run reaching across
 * words (or, for n <= 32, inside one word); the first one found is taken. */
int32_t orc_walk_span(uint32_t *words, uint32_t n_pages, uint32_t n, int32_t seed0,
                      uint32_t max_steps, int32_t *steps);

/* Release n contiguous pages starting at page id (the run may cross words). */
void orc_free_run(uint32_t *words, int32_t id, uint32_t n);
void orc_free_page(uint32_t *words, int32_t id);

/* FIFO free list (linked-list strategy): ring of page ids. */
typedef struct {
    int32_t *ring;       /* capacity entries, -1 = empty */
    uint64_t head, tail; /* tickets */
    int64_t avail;
    uint32_t capacity;
} orc_fifo_t;
void orc_fifo_init(orc_fifo_t *q, int32_t *ring, uint32_t capacity, uint32_t n_free);
int32_t orc_fifo_get(orc_fifo_t *q);
void orc_fifo_put(orc_fifo_t *q, int32_t id);

/* ------------------------------------------------------------------ */
/* Reference-mode replays (pinned against the reference's own outputs)  */
/* ------------------------------------------------------------------ */

/* source/RandomWalkBasic.cuh:54-74 getPage, one thread, int-per-page map. */
int32_t orc_ref_rwbasic_get(int32_t *map, int32_t n_pages, int32_t tid, int16_t clk,
                            int32_t *steps);
/* source/RandomWalkBasic_BM.cuh:60-89 getPage, one thread (returns the
 * reference's id expression verbatim in meaning, quirks included). */
int32_t orc_ref_rwbm_get(int32_t *words, int32_t n_words, int32_t tid, int16_t clk,
                         int32_t *steps);
/* source/CollabRW_BM.cuh:114-160 getPage, one warp with the given active
 * mask, blockIdx.x = block, threadIdx.x = lane. ids/steps per lane. */
void orc_ref_collab_get(int32_t *words, int32_t n_words, uint32_t active, int32_t block,
                        int16_t clk, int32_t *ids, int32_t *steps);
/* source/CRW_BM.cuh:75-142 getPage, one thread. */
int32_t orc_ref_crw_get(int32_t *words, int32_t n_words, int32_t *last_group,
                        int8_t *last_bit, int32_t tid, int16_t clk, int32_t *steps);
/* source/RWMalloc.cuh:159-180 find0Range on one word. */
int32_t orc_ref_find0range(int32_t *x, int32_t *start);
/* source/RWMalloc.cuh:203-248 getNPage, one warp, n[i] pages for lane i. */
void orc_ref_getnpage(int32_t *words, int32_t n_words, int32_t n_pages, uint32_t active,
                      int32_t block, int32_t block_dim, const int32_t *n, int16_t clk,
                      int32_t *ids, int32_t *steps);
/* source/parallelPage.cu:1104-1142 getXPageRandomWalk_BM, one thread. */
int32_t orc_ref_getxpage_rwbm(int32_t *words, int32_t n_words, int32_t X, int32_t tid,
                              int16_t clk, int32_t *steps);
/* source/parallelPage.cu:491-509 getPageSingleClock, one thread. */
int32_t orc_ref_single_clock(int32_t *map, int32_t n_pages, int32_t *arm, int32_t *steps);
/* source/parallelPage.cu:571-592 getPageDistClock, one thread. */
int32_t orc_ref_dist_clock(int32_t *map, int32_t n_pages, int32_t *arms, int32_t tid,
                           int32_t *steps);
/* source/parallelPage.cu:546-555 randomizeArmDistClock for one thread. */
int32_t orc_ref_dist_clock_arm(int32_t tid, int16_t clk, int32_t n_pages);

/* ------------------------------------------------------------------ */
/* CLOCK buffer manager, single-thread replay (oracle_bufmgr.c)        */
/* ------------------------------------------------------------------ */
typedef struct {
    int32_t *page_table;     /* frame or -1 */
    uint64_t *frame_state;   /* (page << 32) | pins */
    uint8_t *ref;
    uint32_t *arms;
    uint64_t hand;
    uint32_t n_logical, n_frames, max_sweep, n_arms;
    int dist;
    uint64_t hits, misses, evictions, failures, unpins, bad_unpins;
} orc_bm_t;
void orc_bm_init(orc_bm_t *b, uint32_t n_logical, uint32_t n_frames, uint32_t max_sweep,
                 uint32_t n_arms, int dist);
void orc_bm_free(orc_bm_t *b);
int32_t orc_bm_fetch(orc_bm_t *b, uint32_t page, uint32_t slot);
void orc_bm_unpin(orc_bm_t *b, int32_t f);
void orc_bm_round(orc_bm_t *b, const int32_t *frames_of, const int32_t *release_idx, uint32_t n_release,
                  const int32_t *pages, uint32_t n, uint32_t slot0, int32_t *frames_out);

/* ------------------------------------------------------------------ */
/* Size-classed malloc, sequential replay (oracle_malloc.c)            */
/* ------------------------------------------------------------------ */
typedef struct {
    uint32_t *words;       /* pool bitmap */
    uint32_t n_pages;
    uint32_t page_shift;
    int32_t *start_of;     /* [n_pages] */
    int32_t *live;         /* [n_pages] */
    uint8_t *len_of;       /* [n_pages] */
} orc_malloc_t;
/* One group of `lanes` requests; offsets[l] = byte offset of the block from
 * the pool base, or -1. */
void orc_malloc_group(orc_malloc_t *m, const uint64_t *sizes, int lanes, int32_t seed_small,
                      const int32_t *seed_own, uint32_t max_steps, int64_t *offsets, int32_t *steps);
/* 1 = freed, 0 = rejected (outside the pool or no live block). */
int orc_malloc_free(orc_malloc_t *m, int64_t offset);

/* Queue-based size classes (oracle_qmalloc.c). */
typedef struct {
    uint32_t *words;
    uint32_t n_pages;
    uint32_t page_shift;
    uint32_t cap;            /* slots per class ring (power of two) */
    uint8_t *class_of;       /* per page: class + 1 (| 0x80 past a chunk's first page) */
    uint32_t *ring;          /* 13 * cap handles (0xffffffff = empty) */
    uint64_t head[13], tail[13];
    int64_t avail[13], space[13];
    uint64_t chunks, overflow, bad_frees;
} orc_qmalloc_t;
int orc_qmalloc_init(orc_qmalloc_t *q, uint32_t *words, uint32_t n_pages, uint32_t page_shift, uint32_t cap);
void orc_qmalloc_destroy(orc_qmalloc_t *q);
void orc_qmalloc_group(orc_qmalloc_t *q, const uint64_t *sizes, int lanes, const int32_t *seed_own,
                       uint32_t max_steps, int64_t *offsets, int32_t *steps);
void orc_qmalloc_free_group(orc_qmalloc_t *q, const int64_t *offsets, int lanes, int32_t *ok);

/* ------------------------------------------------------------------ */
/* std::atomic host replay (CPU baseline), cpu_replay.cpp              */
/* ------------------------------------------------------------------ */
double orc_cpu_churn(uint32_t *words, uint64_t n_pages, int32_t *held, uint64_t n_held,
                     uint64_t n_pairs, uint32_t seed, int threads, int walk, uint32_t max_steps,
                     uint64_t *ok, uint64_t *fail, uint64_t *steps);
double orc_cpu_claim_write_free(uint32_t *words, uint64_t n_pages, uint8_t *pages, uint32_t page_size,
                                uint32_t payload_bytes, uint64_t n, uint32_t seed, int threads, uint32_t reps,
                                uint32_t max_steps, uint64_t *ok, uint64_t *steps);
int orc_hw_threads(void);

#ifdef __cplusplus
}
#endif
#endif
