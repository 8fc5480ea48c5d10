/*
 * pbm.h -- C ABI of the GB300 page and buffer manager (libpbm.so).
 *
 * Plain pointers and sizes only.  Pointers named d_* are device pointers
 * (cudaMalloc'd by the caller), h_* are host pointers, `stream` is a
 * cudaStream_t (NULL = legacy default stream).  Every function returns
 * PBM_OK (0) or a negative status; nothing calls exit() or traps.
 *
 * Each entry point cites the reference interface it replaces.  The
 * reference keeps one implicit pool per translation unit in __device__
 * globals (source/Paging.cuh:37-42, RandomWalkBasic_BM.cuh:28-31); here a
 * pool is an explicit handle, and the reference-named host functions in
 * pbm/ *.cuh bind a per-TU default pool to it.
 */
#ifndef PBM_H
#define PBM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define PBM_OK               0
#define PBM_ERR_INVALID     -1   /* bad argument */
#define PBM_ERR_CUDA        -2   /* a CUDA call failed */
#define PBM_ERR_NOMEM       -3   /* device or host allocation failed */
#define PBM_ERR_EXHAUSTED   -4   /* some requests found no page within their step bound */
#define PBM_ERR_TIMEOUT     -5   /* a bounded device wait gave up */
#define PBM_ERR_UNSUPPORTED -6   /* option not available for this strategy */
#define PBM_ERR_CORRUPT     -7   /* an invariant check failed */

/* ---- allocation strategies (reference names in brackets) ---- */
#define PBM_RANDOM_WALK        0 /* page probe   [getPage, RandomWalkBasic.cuh:54; getPageRandomWalk, parallelPage.cu:152] */
#define PBM_RANDOM_WALK_BM     1 /* word probe   [getPage, RandomWalkBasic_BM.cuh:60; getPageRandomWalk_BM, parallelPage.cu:1066] */
#define PBM_COLLAB_RW_BM       2 /* warp collab  [getPage, CollabRW_BM.cuh:114; getPageCollabRW(_BM), parallelPage.cu:643,830] */
#define PBM_CLUSTERED_RW_BM    3 /* clustered    [getPage, CRW_BM.cuh:75; getPageClusteredRandomWalk(_BM), parallelPage.cu:243,1203] */
#define PBM_LINKED_LIST        4 /* FIFO list    [getPageLinkedList, parallelPage.cu:342] */
#define PBM_SINGLE_CLOCK       5 /* shared arm   [getPageSingleClock, parallelPage.cu:491] */
#define PBM_DIST_CLOCK         6 /* slot arms    [getPageDistClock, parallelPage.cu:571] */
#define PBM_N_STRATEGIES       7

/* ---- batch operations ---- */
#define PBM_OP_ALLOC   0   /* ids[i] <- new page (or -1) */
#define PBM_OP_FREE    1   /* free ids[i] (ids < 0 are skipped) */
#define PBM_OP_SWAP    2   /* allocate a new page, free ids[i], ids[i] <- new page
                              (on failure ids[i] keeps its page) */
#define PBM_OP_MALLOC  3   /* malloc batches: ptrs[i] <- block of sizes[i] bytes (0 on failure) */
#define PBM_OP_MFREE   4   /* malloc batches: free ptrs[i] (0 = nothing), ptrs[i] <- 0 */

/* ---- launch forms ---- */
#define PBM_LAUNCH_PLAIN       0   /* one kernel launch per group */
#define PBM_LAUNCH_PERSISTENT  1   /* one persistent kernel over all groups */
#define PBM_LAUNCH_SERIAL      2   /* malloc batches: one warp, requests in order (deterministic replay) */

/* Pool flags */
#define PBM_POOL_MATERIALIZE   1u  /* also reserve n_pages*page_size bytes of page memory */

typedef struct pbm_pool pbm_pool;

typedef struct {
    uint64_t n_pages;      /* T, 1 .. 2^31-1 */
    uint32_t page_size;    /* bytes per page */
    uint32_t flags;        /* PBM_POOL_* */
    uint32_t max_slots;    /* per-slot walker state (clustered cursors, clock arms); 0 = 1<<22 */
    uint32_t reserved;
} pbm_pool_config;

typedef struct {
    int32_t  strategy;      /* PBM_RANDOM_WALK ... */
    int32_t  word_bits;     /* 32 or 64 (word-probe and collaborative walks) */
    int32_t  collab_width;  /* 8, 16 or 32 lanes per collaborating group; batches also take 64:
                               32 lanes serving two requests each */
    uint32_t stride;        /* words between neighbouring lanes of a collaborating group (>=1) */
    uint32_t max_steps;     /* bound on random jumps per request (0 = 4096) */
    int32_t  block_size;    /* threads per block (0 = 256) */
    int32_t  blocks_per_sm; /* persistent form: resident blocks per SM (0 = occupancy limit;
                               >= 5 selects the register-capped kernels, 5 blocks) */
    int32_t  free_merge;    /* 1 = merge frees of one word within a warp */
    int32_t  fail_fast;     /* pbm_alloc: 1 = count the free pages F before the launch (a pass over
                               the bitmap); requests r >= F fail at once instead of walking to
                               max_steps, the others walk as usual -- or, when the launch asks for
                               at least half of the F pages, request r takes the r-th free page in
                               ascending order (one atomic, no walk) */
    int32_t  reserved;
} pbm_walk_config;

/* One caller's group in a batch.  Requests of the batch are numbered in
 * group order; request q uses LCG seed request_seed(seed, q). */
typedef struct {
    int32_t  op;           /* PBM_OP_* */
    uint32_t count;        /* requests in this group */
    uint64_t offset;       /* first slot of the group in the id arena (wraps at arena_len) */
} pbm_group;

typedef struct {
    uint64_t successes;    /* pages obtained */
    uint64_t failures;     /* requests that hit their step bound */
    uint64_t steps;        /* sum of per-request steps */
    uint64_t frees;        /* pages released */
} pbm_stats;

typedef struct {
    int64_t n_ok, n_failed, n_out_of_range, n_duplicates, n_not_marked;
    int64_t used_pages;    /* popcount of the bitmap after the check */
} pbm_check_result;

/* ---------------- pool ---------------- */

/* initMemoryManagement(nGB, pageSize) [RandomWalkBasic.cuh:39-48, Paging.cuh:59-85],
 * initPages*() [parallelPage.cu:53-71,111-146].  One contiguous reservation
 * instead of 1 GB groups; the bitmap starts all-free. */
int pbm_pool_create(const pbm_pool_config *cfg, pbm_pool **out);
/* (no reference counterpart: the reference never frees its pool) */
int pbm_pool_destroy(pbm_pool *pool);
/* Device addresses and sizes of the pool (bitmap, page memory). */
int pbm_pool_info(const pbm_pool *pool, uint64_t *n_pages, uint32_t *page_size,
                  void **d_bitmap, size_t *bitmap_bytes, void **d_base);
/* resetMemoryManager() [RandomWalkBasic.cuh:86-88]; resetBuffer*() [parallelPage.cu:185-193 ...].
 * Frees every page and resets clock arms, cursors and the free list. */
int pbm_pool_reset(pbm_pool *pool, void *stream);
/* prefillBuffer(freePercentage) [RandomWalkBasic.cuh:121-131]: instead of an
 * allocation run, sets each page held i.i.d. with probability `occupancy`
 * from a counter-based hash of (seed, page). */
int pbm_pool_prefill_bernoulli(pbm_pool *pool, double occupancy, uint64_t seed, void *stream);
/* getFreePagePercentage() [RandomWalkBasic_BM.cuh:117-145], printNumPagesLeft*():
 * number of held pages (popcount of the bitmap); synchronises `stream`. */
int pbm_pool_used(pbm_pool *pool, uint64_t *h_used, void *stream);
/* Snapshot / restore of the bitmap (bytes = bitmap_bytes); synchronous.  A
 * write sets the padding bits past the last page again. */
int pbm_pool_read_bitmap(pbm_pool *pool, void *h_dst, size_t bytes, void *stream);
int pbm_pool_write_bitmap(pbm_pool *pool, const void *h_src, size_t bytes, void *stream);
/* Device addresses of a pool's state, for a caller's own kernels (the
 * drop-in device API in pbm/ *.cuh reads them).  build_fifo != 0 builds the
 * linked-list strategy's free list from the bitmap first.
 * [the reference's __device__ globals set by cudaMemcpyToSymbol,
 * Paging.cuh:69-81, RandomWalkBasic_BM.cuh:47-54, parallelPage.cu:111-146] */
typedef struct {
    void    *words;        /* bitmap, bitmap_bytes */
    void    *base;         /* page memory or NULL */
    uint64_t n_pages;
    uint32_t page_size;
    uint32_t n_words32;
    uint32_t n_words64;
    uint32_t max_slots;    /* entries of cursors / arms */
    void    *cursors;      /* int32[max_slots]: clustered walk, last page per slot (-1 = none) */
    void    *arms;         /* uint32[max_slots]: distributed clock arms */
    void    *single_arm;   /* unsigned long long: single clock arm */
    void    *fifo_state;   /* free-list tickets (see pbm/pbm_device.cuh FifoState) */
    void    *fifo_ring;    /* int32[n_pages] free-list ring, NULL until built */
    void    *stats;        /* device statistics block */
} pbm_device_state;
int pbm_pool_device_state(pbm_pool *pool, int build_fifo, pbm_device_state *h_out, void *stream);
/* Accumulated device statistics since create/reset (synchronises `stream`). */
int pbm_pool_stats(pbm_pool *pool, pbm_stats *h_out, void *stream);

/* ---------------- page allocation ---------------- */

/* n requests, one page each: d_ids[i] <- page or -1, d_steps[i] <- steps
 * (d_steps may be NULL).  [getPage*(int*) from every strategy, launched as
 * the reference's drivers do, e.g. get1page_kernel, unitTest1.cu:22-30] */
int pbm_alloc(pbm_pool *pool, const pbm_walk_config *cfg, uint32_t n, uint32_t seed,
              int32_t *d_ids, int32_t *d_steps, void *stream);
/* Same requests processed in order by one thread (one warp for the
 * collaborative walk): a deterministic replay. */
int pbm_alloc_serial(pbm_pool *pool, const pbm_walk_config *cfg, uint32_t n, uint32_t seed,
                     int32_t *d_ids, int32_t *d_steps, void *stream);
/* freePage*(pageID) [RandomWalkBasic.cuh:82-84, RandomWalkBasic_BM.cuh:98-102,
 * parallelPage.cu:180,265,...]: ids < 0 are skipped. */
int pbm_free(pbm_pool *pool, const pbm_walk_config *cfg, uint32_t n, const int32_t *d_ids,
             void *stream);
/* Contiguous runs: d_npages[i] pages (1..32) inside one bitmap word.
 * [getXPageRandomWalk_BM, parallelPage.cu:1104-1142; getNPage, RWMalloc.cuh:203-248] */
int pbm_alloc_runs(pbm_pool *pool, uint32_t n, const int32_t *d_npages, uint32_t seed,
                   uint32_t max_steps, int32_t *d_ids, int32_t *d_steps, void *stream);
int pbm_alloc_runs_serial(pbm_pool *pool, uint32_t n, const int32_t *d_npages, uint32_t seed,
                          uint32_t max_steps, int32_t *d_ids, int32_t *d_steps, void *stream);
/* Runs of d_npages[i] pages (1 .. 65536) that may cross word boundaries,
 * which lifts the one-word limit of the reference's contiguous claims: per
 * jump the walk scans from a random word for a free run reaching across
 * words (for runs of <= 32 pages also inside one word) and claims it word by
 * word, releasing its bits again if another claim took part of it.
 * [getXPage*_BM, parallelPage.cu:934-991, 1104-1142; getNPage, RWMalloc.cuh:113-157,
 * without their single-word restriction] */
int pbm_alloc_spans(pbm_pool *pool, uint32_t n, const int32_t *d_npages, uint32_t seed,
                    uint32_t max_steps, int32_t *d_ids, int32_t *d_steps, void *stream);
int pbm_alloc_spans_serial(pbm_pool *pool, uint32_t n, const int32_t *d_npages, uint32_t seed,
                           uint32_t max_steps, int32_t *d_ids, int32_t *d_steps, void *stream);
/* Releases d_npages[i] pages from d_ids[i] on (1 .. 65536 pages, runs from
 * either claim form; entries with an id < 0 or past the pool are skipped).
 * [releasePages, CollabRW_BM.cuh:61-71; freeRW, RWMalloc.cuh:329-334] */
int pbm_free_runs(pbm_pool *pool, uint32_t n, const int32_t *d_ids, const int32_t *d_npages,
                  void *stream);

/* The page-pool workload of the reference's drivers: each of n requests
 * claims one page (page-probe walk), writes its request index into the
 * first payload_bytes of the page and frees it again unless `hold`.
 * Needs a pool created with PBM_POOL_MATERIALIZE.
 * [get1page_kernel + freePage_kernel, unitTest1.5.cu:127-150; getPagePtr,
 * RandomWalkBasic.cuh:76-79] */
int pbm_claim_write_free(pbm_pool *pool, uint32_t n, uint32_t seed, uint32_t payload_bytes, int hold,
                         uint32_t max_steps, int32_t *d_ids, int32_t *d_steps, void *stream);
/* Copies the first bytes_per_page bytes of each listed page into d_out
 * (n * bytes_per_page bytes; ids < 0 give zeros).  [pageAddress, Paging.cuh:30-38] */
int pbm_gather_pages(pbm_pool *pool, const int32_t *d_ids, uint32_t n, uint32_t bytes_per_page,
                     int32_t *d_out, void *stream);

/* ---------------- batches ---------------- */

/* Runs the groups of one batch.  d_groups: device array of n_groups
 * descriptors; h_groups: the same descriptors in host memory (needed by the
 * plain form, which launches one kernel per group; may be NULL for the
 * persistent form).  d_arena: id arena of arena_len slots.  The persistent
 * form is a single launch and can be captured in a CUDA graph.
 * Persistent form with d_groups NULL: the host table h_groups (at most
 * PBM_MAX_INLINE_GROUPS groups) is copied into the launch's parameters, so the
 * step needs no separate host-to-device copy; h_groups may be reused as soon
 * as the call returns. */
#define PBM_MAX_INLINE_GROUPS 256
int pbm_batch_launch(pbm_pool *pool, const pbm_walk_config *cfg, const pbm_group *d_groups,
                     const pbm_group *h_groups, uint32_t n_groups, int32_t *d_arena,
                     uint64_t arena_len, uint32_t seed, int32_t *d_steps, int mode, void *stream);
/* The same, also writing each request's result to results[q] (request
 * order q = 0 .. total-1): the new page of an ALLOC or SWAP (-1 if none was
 * found), the page a FREE released.  `results` may be host memory mapped into
 * the device (pinned, e.g. cudaHostAlloc): the kernel then streams the step's
 * results to the host over the chip-to-chip link while it runs, with no
 * separate device-to-host copy.  Pageable (unregistered) host memory is
 * refused with PBM_ERR_INVALID before anything is launched.  (No reference
 * counterpart.) */
int pbm_batch_launch_results(pbm_pool *pool, const pbm_walk_config *cfg, const pbm_group *d_groups,
                             const pbm_group *h_groups, uint32_t n_groups, int32_t *d_arena, uint64_t arena_len,
                             uint32_t seed, int32_t *d_steps, int32_t *results, int mode, void *stream);

/* Graph-replayed persistent batch.  Replay k reads the descriptors at
 * d_groups + (k mod n_steps)*n_groups with seed seed0 + k.  The batch graph
 * counts its replays on the host: pbm_graph_replay writes k into the graph's
 * kernel parameters before it launches (launches already queued keep their
 * own k) and advances it; pbm_graph_set_step sets it.  Replay any number of
 * times, from one host thread at a time and in stream order.  (The malloc
 * graphs keep their counter in device memory and advance it with a kernel of
 * the graph.) */
typedef struct pbm_graph pbm_graph;
int pbm_batch_graph_create(pbm_pool *pool, const pbm_walk_config *cfg, const pbm_group *d_groups,
                           uint32_t n_groups, uint32_t n_steps, int32_t *d_arena,
                           uint64_t arena_len, uint32_t seed0, void *stream, pbm_graph **out);
/* The graph form of pbm_batch_launch_results: each replay also writes its
 * step's results to results[q] (device or pinned host memory). */
int pbm_batch_graph_create_results(pbm_pool *pool, const pbm_walk_config *cfg, const pbm_group *d_groups,
                                   uint32_t n_groups, uint32_t n_steps, int32_t *d_arena, uint64_t arena_len,
                                   uint32_t seed0, int32_t *results, void *stream, pbm_graph **out);
int pbm_graph_replay(pbm_graph *g, void *stream);
int pbm_graph_set_step(pbm_graph *g, uint32_t step, void *stream);
int pbm_graph_destroy(pbm_graph *g);

/* ---------------- size-classed malloc over the pool's pages ----------------
 * [mallocRW / freeRW, RWMalloc.cuh:299-334; MemoryManager::malloc / free,
 * malloc.cuh:3-37, malloc.cu:223-320].  Sizes round up to power-of-two
 * classes 16 B .. 64 KiB; the sub-page requests of each group of 32
 * consecutive requests share one run of pages (largest class first, so each
 * sub-page block is aligned to its size); larger requests take their own
 * run and start on a page boundary; the
 * last free of a run releases it.  Needs a materialised pool with a
 * power-of-two page size in 2 KiB .. 64 KiB. */
int pbm_malloc_init(pbm_pool *pool);     /* side tables: 9 bytes per page */
int pbm_malloc_release(pbm_pool *pool);
/* Device addresses of the malloc side tables (int32 start_of[T], int32
 * live[T], uint8 len_of[T]) for a caller's own kernels (pbm/pbm_malloc.cuh). */
int pbm_malloc_tables(pbm_pool *pool, void **d_start_of, void **d_live, void **d_len_of);
/* Groups use PBM_OP_MALLOC / PBM_OP_MFREE; slot i of a group is arena slot
 * (offset + i) mod arena_len of d_sizes (uint32 bytes) and d_ptrs (device
 * addresses).  mode: PBM_LAUNCH_PLAIN (h_groups needed), _PERSISTENT or _SERIAL. */
int pbm_malloc_batch(pbm_pool *pool, const pbm_group *d_groups, const pbm_group *h_groups, uint32_t n_groups,
                     const uint32_t *d_sizes, unsigned long long *d_ptrs, uint64_t arena_len, uint32_t seed,
                     uint32_t max_steps, int mode, void *stream);
/* Graph form: replay k reads d_groups + (k mod n_steps)*n_groups with seed seed0 + k. */
int pbm_malloc_graph_create(pbm_pool *pool, const pbm_group *d_groups, uint32_t n_groups, uint32_t n_steps,
                            const uint32_t *d_sizes, unsigned long long *d_ptrs, uint64_t arena_len,
                            uint32_t seed0, uint32_t max_steps, void *stream, pbm_graph **out);
/* Runs still holding blocks, and frees rejected so far (outside the pool or
 * double frees); synchronous. */
int pbm_malloc_counts(pbm_pool *pool, uint64_t *h_live_runs, uint64_t *h_bad_frees, void *stream);

/* ---------------- queue-based size classes (no reference counterpart) ----------------
 * The same malloc / free batches over a second backend: per size class a
 * bounded FIFO ring of free blocks, as the page queues of the allocator the
 * reference vendors as its comparator (Ouroboros,
 * source/Ouroboros/include/device/queues/page/PageQueueVL_impl.cuh).  Lanes of
 * a warp that ask for one class take blocks with one reservation; lanes the
 * ring cannot serve carve chunks (one page for classes below a page, one block
 * above) from the pool with the spanning walk and enqueue the blocks nobody
 * took; frees go back to their class's ring.  Chunks stay with their class
 * until release.  ring_capacity: blocks per class ring (power of two,
 * 0 = 2^20); a free into a full ring drops the block (counted).  Pools up to
 * 64 GiB (32-bit handles of 16 bytes); needs PBM_POOL_MATERIALIZE.  Frees are
 * not checked for doubles. */
int pbm_qmalloc_init(pbm_pool *pool, uint32_t ring_capacity);
int pbm_qmalloc_release(pbm_pool *pool);
int pbm_qmalloc_batch(pbm_pool *pool, const pbm_group *d_groups, const pbm_group *h_groups, uint32_t n_groups,
                      const uint32_t *d_sizes, unsigned long long *d_ptrs, uint64_t arena_len, uint32_t seed,
                      uint32_t max_steps, int mode, void *stream);
int pbm_qmalloc_graph_create(pbm_pool *pool, const pbm_group *d_groups, uint32_t n_groups, uint32_t n_steps,
                             const uint32_t *d_sizes, unsigned long long *d_ptrs, uint64_t arena_len,
                             uint32_t seed0, uint32_t max_steps, void *stream, pbm_graph **out);
/* h_queued[13]: blocks waiting in each class ring (16 B .. 64 KiB); chunks
 * carved so far; blocks dropped by full rings; bounded waits that gave up;
 * frees rejected (outside the pool, not at a block start, no chunk). */
int pbm_qmalloc_counts(pbm_pool *pool, uint64_t *h_queued, uint64_t *h_chunks, uint64_t *h_overflow,
                       uint64_t *h_timeouts, uint64_t *h_bad_frees, void *stream);

/* Autotuner (no reference counterpart).  Runs the caller's batch of
 * `requests` swap requests (descriptors in d_groups, all PBM_OP_SWAP) through
 * the persistent kernel for every candidate configuration -- walk, width
 * 8/16/32, 32/64-bit words, stride, blocks per SM, merged frees -- once
 * untimed and then `reps` times, each timed alone after an L2 flush (a
 * 256 MiB device scratch, allocated for the call), ranked by the median
 * (ms_per_batch) and, where medians tie (event timings are quantised), by
 * the mean (ms_mean); candidates that tie on both keep the candidate order.
 * Returns up to max_out results sorted fastest first.  Swaps keep the pool's
 * occupancy, so tune once per occupancy band. */
typedef struct {
    pbm_walk_config cfg;
    float ms_per_batch;    /* median of the reps */
    float ms_mean;         /* mean of the reps */
    double ops_per_s;      /* 2 * requests / time (one alloc + one free each) */
} pbm_tune_result;
int pbm_autotune(pbm_pool *pool, const pbm_group *d_groups, uint32_t n_groups, uint64_t requests,
                 int32_t *d_arena, uint64_t arena_len, uint32_t seed, int reps, uint32_t max_steps,
                 pbm_tune_result *h_out, uint32_t max_out, uint32_t *h_n_out, void *stream);

/* ---------------- buffer manager with CLOCK replacement ----------------
 * No reference counterpart: the reference's "_BM" files are bitmap
 * allocators; its SingleClock / DistClock arms (parallelPage.cu:491-509,
 * 571-592) sweep a free map.  Here the same sweeps choose eviction victims
 * for a page table over n_logical pages cached in n_frames frames.  A fetch
 * pins the frame it returns until pbm_bufmgr_round releases it. */
#define PBM_BM_SINGLE_CLOCK 0   /* one shared hand */
#define PBM_BM_DIST_CLOCK   1   /* n_arms private hands, request i uses arm (slot0 + i) % n_arms */

typedef struct pbm_bufmgr pbm_bufmgr;
typedef struct {
    uint64_t n_logical;    /* logical pages (page-table entries) */
    uint32_t n_frames;     /* buffer frames */
    uint32_t frame_size;   /* bytes per frame (multiple of 16; 0 = metadata only) */
    int32_t  policy;       /* PBM_BM_SINGLE_CLOCK or PBM_BM_DIST_CLOCK */
    uint32_t n_arms;       /* hands of the distributed clock (0 = 1) */
    uint32_t max_sweep;    /* hand steps before a miss gives up (0 = 2*n_frames + 64) */
    uint32_t reserved;
} pbm_bufmgr_config;

typedef struct {
    uint64_t hits, misses, evictions, failures, unpins, bad_unpins, timeouts;
} pbm_bufmgr_counters;

typedef struct {
    uint64_t resident;       /* page-table entries that point at a frame */
    uint64_t mapped_frames;  /* frames holding a page */
    uint64_t mismatches;     /* entries whose frame does not point back */
    uint64_t loading;        /* pages left half-loaded */
    uint64_t pins;           /* total pins held */
} pbm_bufmgr_check_result;

/* d_backing: n_logical * frame_size bytes copied into a frame on each miss
 * (NULL = no copy). */
int pbm_bufmgr_create(const pbm_bufmgr_config *cfg, const void *d_backing, pbm_bufmgr **out);
int pbm_bufmgr_destroy(pbm_bufmgr *m);
int pbm_bufmgr_reset(pbm_bufmgr *m, void *stream);
/* One round: unpin d_frames_of[d_release_idx[j]] for j < n_release, then
 * fetch d_pages[0..n) into d_frames_out (-1 = no frame).  Request i of the
 * round uses distributed-clock arm (slot0 + i) % n_arms.  serial != 0: one
 * thread, releases then fetches in order (deterministic replay).  In the
 * parallel form a round's releases may land after other fetches of the same
 * round (a sweep passes a page whose release has not landed as pinned).  A
 * page holds at most 2^30 - 1 pins at a time.  A release of a pin that is not
 * held is counted bad and undone; until it is undone, a fetch of the same
 * page may see it as pinned or, if the page is not resident, wait for it.
 * Releases of one frame (or page) in the same block of the launch (in the
 * same warp for a round of releases only) merge into one release, which is
 * rejected whole if it asks for more pins than are held.
 * A round with releases and no fetches (n = 0) only unpins: the clock hand
 * and the reference bits stay as they were. */
int pbm_bufmgr_round(pbm_bufmgr *m, const int32_t *d_frames_of, const int32_t *d_release_idx,
                     uint32_t n_release, const int32_t *d_pages, uint32_t n, uint32_t slot0,
                     int32_t *d_frames_out, int serial, void *stream);
/* The same round with pins released by page, as a buffer pool's
 * unpin(page) names them: unpin page d_pages_of[d_release_idx[j]] for
 * j < n_release (negative entries are skipped), then fetch d_pages[0..n) into
 * d_frames_out.  A release then needs no frame-to-page lookup.  d_held_out
 * (may be NULL) receives, for each fetch, its page if it pinned a frame and
 * -1 if it did not: an array that later rounds' release lists can name, so
 * that no release names a fetch that holds nothing. */
int pbm_bufmgr_round_pages(pbm_bufmgr *m, const int32_t *d_pages_of, const int32_t *d_release_idx,
                           uint32_t n_release, const int32_t *d_pages, uint32_t n, uint32_t slot0,
                           int32_t *d_frames_out, int32_t *d_held_out, int serial, void *stream);
int pbm_bufmgr_stats(pbm_bufmgr *m, pbm_bufmgr_counters *h_out, void *stream);
int pbm_bufmgr_check(pbm_bufmgr *m, pbm_bufmgr_check_result *h_out, void *stream);
int pbm_bufmgr_frames(pbm_bufmgr *m, void **d_frames, size_t *bytes);
/* Copies the maps to the host (either pointer may be NULL; synchronises
 * `stream`): h_page_entries[n_logical], one 64-bit word per logical page --
 * the frame holding it in the high 32 bits (signed: -1 not resident, -2 and
 * -3 a load in progress), the CLOCK reference bit in bit 31, a guard bit
 * (bit 30, set while no release is being undone), its pins in bits 0..29; h_frame_pages[n_frames], the page each frame holds
 * (0xffffffff empty).  No reference counterpart. */
int pbm_bufmgr_read_tables(pbm_bufmgr *m, uint64_t *h_page_entries, uint32_t *h_frame_pages, void *stream);
/* Copies the first bytes_per_frame bytes of each listed frame into d_out
 * (ids < 0 give zeros). */
int pbm_bufmgr_gather(pbm_bufmgr *m, const int32_t *d_frame_ids, uint32_t n, uint32_t bytes_per_frame,
                      int32_t *d_out, void *stream);

/* ---------------- serving loop (no reference counterpart) ----------------
 * Continuous batching of many tenants' requests over one resident pool (and
 * buffer manager for fetches).  pbm_server_run replays the requests in real
 * time from their arrival stamps (seconds from the start of the run, sorted).
 * ALLOC n: n new pages appended to the tenant's ring of page slots.
 * FREE n:  releases min(n, pages the tenant holds) of its oldest pages.
 * FETCH n: pins then releases the next n pages of the shared fetch trace.
 * Admission is by a free-page budget shared by all tenants: the pages free
 * below max_occupancy at create time.  An ALLOC that does not fit the budget
 * now waits until frees land (frees count once their batch has finished);
 * only an ALLOC larger than the budget, the tenant's ring or its optional
 * quota is rejected (status PBM_ERR_EXHAUSTED).  A tenant's ALLOCs keep
 * their arrival order; a later FREE may pass a waiting ALLOC when all the
 * pages it releases are older than that ALLOC, a FETCH always may.  A FREE
 * waits until the pages it releases are allocated on the device.  Admitted
 * requests of all tenants form the next batch whenever one of n_streams
 * batch slots is free, so batches overlap on the device.  A request's status
 * and page count depend only on its tenant's own requests, so they are the
 * same alone and in a mix for every request the mix admits; when nothing is
 * left to arrive or run and nothing more can be admitted, the run stops and
 * the requests still waiting end with status -1 (counted as stranded). */
#define PBM_REQ_ALLOC 0
#define PBM_REQ_FREE  1
#define PBM_REQ_FETCH 2

typedef struct {
    double   arrival_s;
    uint32_t tenant;
    int32_t  op;           /* PBM_REQ_* */
    uint32_t count;        /* pages */
    uint32_t reserved;
} pbm_request;

typedef struct {
    double   admit_s, launch_s, done_s, latency_s;   /* seconds since the run started */
    uint64_t pages;        /* pages allocated / released / fetched */
    int32_t  status;       /* 0 done, PBM_ERR_EXHAUSTED over budget, -1 never admitted */
    uint32_t reserved;
} pbm_request_result;

typedef struct {
    uint32_t n_tenants;
    uint32_t ring_pages;          /* page slots per tenant */
    uint32_t n_streams;           /* batches in flight at most */
    uint32_t max_batch_requests;  /* requests per batch at most (<= 2048) */
    uint32_t max_fetch_pages;     /* fetch pages per batch at most (0 = 1<<22) */
    uint32_t tenant_quota_pages;  /* pages one tenant may hold (0 = no cap beyond the shared budget) */
    double   max_occupancy;       /* bound on held pages / pool pages (sets the shared budget) */
    double   drain_timeout_s;     /* stop waiting this long after the last arrival */
    pbm_walk_config walk;         /* allocation walk of the batches */
} pbm_server_config;

typedef struct {
    uint64_t requests, completed, rejected, pages, batches, max_in_flight;
    double   wall_s, p50_s, p99_s, mean_batch_requests;
    uint64_t waited;      /* ALLOCs that waited for memory before admission */
    uint64_t stranded;    /* requests still waiting when the run stopped (status -1) */
} pbm_server_report;

typedef struct pbm_server pbm_server;
/* bm may be NULL when no request fetches; d_fetch_pages: logical page ids. */
int pbm_server_create(pbm_pool *pool, pbm_bufmgr *bm, const int32_t *d_fetch_pages, uint64_t n_fetch_pages,
                      const pbm_server_config *cfg, pbm_server **out);
int pbm_server_run(pbm_server *s, const pbm_request *h_reqs, uint64_t n, pbm_request_result *h_results,
                   pbm_server_report *h_report);
/* Pages a tenant holds now, oldest first (h_out may be NULL to get the count). */
int pbm_server_tenant_pages(pbm_server *s, uint32_t tenant, int32_t *h_out, uint64_t max_out, uint64_t *h_n);
int pbm_server_destroy(pbm_server *s);

/* ---------------- monitor: occupancy sampled while kernels run ----------------
 * [monitorBufferRandomWalk, parallelPage.cu:209-223, as a host-polled
 * sampler]  A host thread samples the pool every interval_us on its own
 * non-blocking stream (a popcount kernel over the bitmap and a copy of the
 * statistics block) until max_samples or pbm_monitor_stop; its kernel fits
 * beside the pool's persistent kernels, so samples are taken while they run.
 * The pool must outlive the monitor. */
typedef struct {
    double   t_s;            /* seconds since pbm_monitor_start */
    uint64_t used_pages;
    double   free_fraction;
    pbm_stats stats;         /* the pool's counters at that time */
} pbm_monitor_sample;
typedef struct pbm_monitor pbm_monitor;
int pbm_monitor_start(pbm_pool *pool, uint32_t interval_us, uint32_t max_samples, pbm_monitor **out);
/* Copies up to max_out samples taken so far; *h_n = samples taken. */
int pbm_monitor_samples(pbm_monitor *m, pbm_monitor_sample *h_out, uint32_t max_out, uint32_t *h_n);
int pbm_monitor_stop(pbm_monitor *m);

/* ---------------- checks and measurement ---------------- */

/* Invariants of an allocation result: ids in range, no page handed to two
 * requesters, every returned page marked held; plus the pool's popcount. */
int pbm_check_ids(pbm_pool *pool, const int32_t *d_ids, uint32_t n, pbm_check_result *h_out,
                  void *stream);

/* The same invariant check for callers that cannot allocate device memory
 * (no counterpart in the reference).  An engine that gives all of its device
 * memory to its own buffer pool at start-up, or a process that must not grow
 * its device footprint after start-up, has the bitmap and the id list already
 * but no way to get scratch.  This entry point calls no cudaMalloc/cudaFree:
 * its scratch (one bit per page plus counters) is a static device array of
 * 1 MiB + 128 B that every GPU loading libpbm.so keeps until exit, so it
 * accepts at most 8,388,608 pages and INT32_MAX ids (PBM_ERR_INVALID beyond).
 * d_bitmap uses the pool layout (bit p of 32-bit word p/32 = page p held).
 * All calls share the scratch and each call clears it first: calls that
 * overlap on the GPU race, so serialise them.  The call waits for `stream`
 * before it returns.  The first call on a device (and again after a device
 * reset) resolves the scratch address (cudaGetSymbolAddress), so make it
 * before any stream capture. */
int pbm_check_ids_noalloc(const uint32_t *d_bitmap, uint64_t n_pages, const int32_t *d_ids,
                          uint32_t n, pbm_check_result *h_out, void *stream);

/* Uncontended atomicOr ceiling (the roofline denominator of the allocation
 * kernels): `threads` threads each issue `iters` atomicOr operations
 * (returning = 1: the old value is used) on words no other thread touches in
 * the same iteration, in a `words`-word buffer.  pattern 1 = the 32 lanes of
 * a warp hit one 128-byte line, 2 = lanes 33 words apart (32 lines per warp
 * instruction), 0 = the faster of the two.  h_ops_per_s <- RMW/s from CUDA
 * events (best of 5).  [precedent: unitTestLinkedList2.cu:3-16] */
int pbm_atomic_ceiling(uint32_t words, uint32_t threads, uint32_t iters, int returning, int pattern,
                       double *h_ops_per_s, double *h_ms);

/* Library identity and the number of kernels this library has launched. */
const char *pbm_version(void);
uint64_t pbm_kernel_launches(void);
int pbm_device_sm_count(int *h_sms);

#ifdef __cplusplus
}
#endif
#endif /* PBM_H */
